/*
 * hasty_gpu.h - C ABI of the GB300 path tracer.
 *
 * A drop-in for HastyRenderer's unidirectional CPU integrator behind the
 * reference's render-job surface. Plain C types only; every call returns an
 * int status (HASTY_OK or a negative HASTY_ERR_*) and never throws. The
 * message of the calling thread's last failure is available through
 * hasty_last_error().
 *
 * Reference interfaces replaced (paths relative to the reference project):
 *   hasty_job_load           RenderJob::loadJSON + Scene::Scene
 *                            (core/src/RenderJob.cpp:21-28, core/src/Scene.cpp:12-194)
 *   hasty_job_render_passes  renderThread pass loop over estimateRadiance
 *                            (core/src/PathTracing.cpp:98-160, :21-95)
 *   hasty_job_stop           RenderJob::stopFlag (core/include/Hasty/RenderJob.h:51)
 *   hasty_job_read           computeEstimate (apps/ViewerUtils.cpp:95-121)
 *   hasty_job_write_outputs  postProcessAndSaveToDisk without the denoiser
 *                            (apps/ViewerUtils.cpp:137-152)
 *   hasty_debug_intersect    Scene::rayHit / rtcIntersect1 (core/src/Scene.cpp:281-303)
 *   hasty_debug_bsdf         PrincipledBRDF::sample / evaluate / evaluateSamplePDF
 *                            (core/src/BRDF.cpp:630-742)
 *
 * Threading: a context and its jobs may be used from one host thread at a
 * time. Rendering is asynchronous on the job's CUDA stream; hasty_job_sync,
 * hasty_job_read and hasty_job_write_outputs wait for it.
 */
#ifndef HASTY_GPU_H
#define HASTY_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HASTY_OK 0
#define HASTY_ERR_ARG (-1)        /* bad argument (CLI exit code 1) */
#define HASTY_ERR_LOAD (-2)       /* job/scene/mesh/image could not be loaded (CLI exit code 2) */
#define HASTY_ERR_CUDA (-3)       /* CUDA runtime error or no device */
#define HASTY_ERR_MEMORY (-4)     /* device allocation failed */
#define HASTY_ERR_IO (-5)         /* output could not be written (CLI exit code 5) */
#define HASTY_ERR_STOPPED (-6)    /* job was stopped before the requested passes ran */
#define HASTY_ERR_MISSING (-7)    /* entry point not compiled into the library */

/* hasty_ctx_create flags */
#define HASTY_CTX_BINARY_BVH 1u   /* binary BVH instead of the compressed 8-wide one */
#define HASTY_CTX_HOST_BVH 2u     /* build the BVH on the host instead of the GPU */
#define HASTY_CTX_WAVEFRONT 4u    /* never the path kernel (every scene on the wavefront kernels) */
#define HASTY_CTX_PATH_KERNEL 8u  /* the path kernel for every scene (default: the wavefront, or the
                                   * path kernel for scenes of at most HASTY_PATH_KERNEL_TRIS triangles) */

#define HASTY_AOV_COLOR 0
#define HASTY_AOV_NORMAL 1
#define HASTY_AOV_ALBEDO 2

typedef struct hasty_ctx hasty_ctx;
typedef struct hasty_job hasty_job;

typedef struct hasty_job_info {
  int32_t width, height;
  int32_t num_samples;         /* settings.num_samples */
  int32_t max_depth;
  int32_t roulette_start_depth;
  float roulette_q;
  int32_t use_mis;
  uint64_t seed;
  int64_t n_triangles;
  int64_t n_light_triangles;
  int32_t n_shapes;
  int32_t n_materials;
  int32_t env_is_texture;
  float exposure;
  int32_t samples_done;        /* passes accumulated so far */
  int32_t bvh_depth;
  double bvh_build_ms;
  int64_t device_bytes;        /* device memory held by the job */
  double bvh_tree_ms;          /* part of bvh_build_ms spent building the binary tree */
  double parse_ms;             /* job load: renderJob/scene JSON, OBJ/MTL and images read on the host */
  double upload_ms;            /* job load: host-to-device copies of the scene (after the BVH build) */
  int64_t paths_in_flight;     /* camera samples per batch at most (whole passes) */
  int32_t path_kernel;         /* 1: rendered by the path kernel (cache-resident scene), 0: the wavefront */
  int32_t pad;
} hasty_job_info;

typedef struct hasty_stats {
  uint64_t rays;               /* closest-hit queries (camera, BSDF and light rays) */
  uint64_t shaded;             /* non-emissive surface vertices shaded */
  uint64_t paths;              /* camera samples started */
  uint64_t nan_samples;        /* samples dropped for NaN radiance */
  uint64_t media_overflow;     /* medium-stack pushes dropped (beyond 20 nested media) */
  uint64_t trial_cap;          /* rejection loops stopped at the trial limit */
  double kernel_ms;            /* device time of the passes rendered so far */
  double trace_ms;             /* device time in closest-hit kernels (stage timing on) */
  double shade_ms;             /* device time in shading kernels (stage timing on) */
  uint64_t trace_launches;     /* closest-hit kernel launches */
  uint64_t kernel_launches;    /* all kernel launches of the passes rendered so far */
  double path_ms;              /* device time in the path kernel (stage timing on) */
  uint64_t path_launches;      /* path-kernel launches */
  uint64_t stack_overflow;     /* rays whose BVH traversal stack overflowed (a subtree skipped) */
} hasty_stats;

int hasty_last_error(char* buf, size_t len);
int hasty_version(int* major, int* minor);

int hasty_ctx_create(int device, uint32_t flags, hasty_ctx** out);
int hasty_ctx_destroy(hasty_ctx* ctx);

int hasty_job_load(hasty_ctx* ctx, const char* render_job_path, hasty_job** out);
/* Loads n jobs as hasty_job_load would, on `threads` host threads at once
 * (0: as many as the host has, at most n): parse, BVH build and upload of
 * different jobs overlap. out[i] receives job i. All or nothing: on the first
 * failure no job is returned (out[] is left null) and the status and
 * hasty_last_error are that job's. For a batch or server front end that
 * starts from many renderJob files (no reference counterpart: the reference
 * loads one job per process, apps/PathTracingViewer.cpp:34-37). */
int hasty_jobs_load(hasty_ctx* ctx, const char* const* render_job_paths, size_t n, int32_t threads, hasty_job** out);
int hasty_job_destroy(hasty_job* job);
int hasty_job_info_get(hasty_job* job, hasty_job_info* out);
int hasty_job_set_seed(hasty_job* job, uint64_t seed);      /* also clears the accumulators */
int hasty_job_reset(hasty_job* job);                        /* clears accumulators, pass counter, stats */
/* Maximum camera samples in flight per batch (paths); 0 = automatic. */
int hasty_job_set_paths_in_flight(hasty_job* job, int64_t paths);

/* Frees the job's path state (re-allocated by the next render); synchronous. */
int hasty_job_release_paths(hasty_job* job);

int hasty_job_render_passes(hasty_job* job, int n_passes);  /* asynchronous */
int hasty_job_sync(hasty_job* job);
int hasty_job_stop(hasty_job* job);
int hasty_job_stats_get(hasty_job* job, hasty_stats* out);
/* Time every stage with CUDA events (adds two events per kernel). */
int hasty_job_set_stage_timing(hasty_job* job, int on);

/* Estimate sum / (1e-7 + N); colour scaled by 2^exposure. host_rgb holds w*h*3 floats, row-major. */
int hasty_job_read(hasty_job* job, int aov, float* host_rgb, size_t w, size_t h, int32_t* num_samples);
/* Raw FP64 sums over the passes rendered so far (w*h*3 doubles). */
int hasty_job_read_sums(hasty_job* job, int aov, double* host_rgb, size_t w, size_t h, int32_t* num_samples);
/* output.exr, outputNormal.exr, outputAlbedo.exr (+ .pfm copies when write_pfm != 0). */
int hasty_job_write_outputs(hasty_job* job, const char* out_dir, int write_pfm);

/* ---- Progressive read-back while rendering continues ---------------------
 * The reference's viewer shows computeEstimate of the colour buffers every
 * ~20 ms while its render threads run (apps/PathTracingViewer.cpp:88-139,
 * apps/ViewerUtils.cpp:95-121) and saves the three estimates at the end
 * (:157-172). Here a snapshot computes the estimates of the AOVs in aov_mask
 * (bit 1 << HASTY_AOV_*) behind every pass enqueued so far and copies them
 * into pinned host memory on a copy stream; the call returns at once and
 * passes enqueued afterwards do not wait for the copy.
 *
 *   hasty_job_snapshot        enqueue a snapshot (replaces the previous one)
 *   hasty_job_snapshot_query  *ready = 1 once its copy has landed (no wait)
 *   hasty_job_snapshot_get    wait for it; *out = w*h*3 floats of `aov`
 *                             (colour x 2^exposure), valid until the next
 *                             hasty_job_snapshot; *num_samples = passes covered
 *   hasty_job_write_outputs_async  the files of hasty_job_write_outputs from
 *                             a snapshot of this moment, written by a host
 *                             thread (a previous write is waited for first)
 *   hasty_job_outputs_wait    wait for that write and return its status
 */
int hasty_job_snapshot(hasty_job* job, uint32_t aov_mask);
int hasty_job_snapshot_query(hasty_job* job, int* ready);
int hasty_job_snapshot_get(hasty_job* job, int aov, const float** out, int32_t* num_samples);
int hasty_job_write_outputs_async(hasty_job* job, const char* out_dir, int write_pfm);
int hasty_job_outputs_wait(hasty_job* job);

/* ---- Photon mapping (the reference's second integrator) ------------------
 * Stochastic progressive photon mapping with a caustics map, as one render
 * thread of the reference runs it (core/src/PhotonMapping.cpp:814-935,
 * renderPhotonThread; PMRenderJob, core/include/Hasty/PhotonMapping.h): per
 * iteration, photons from the area lights (sampleLightRay) are traced until
 * 0.5*W*H caustic photons (L S+ D, stored at diffuse surfaces after the first
 * bounce) are stored or 10*W*H were emitted; every pixel then path-traces
 * with both MIS strategies, adds photon estimates at diffuse vertices (hash
 * cells, per-pixel radius) and updates its radius/flux statistics (alpha
 * 0.4). Initial radii: 10x the pixel footprint with a surface light, else 1.
 * Random streams are keyed per photon and per pixel (the reference shares
 * one stream per thread), so results do not depend on threads. Replaces the
 * render threads of apps/PhotonMappingViewer.cpp:48-57. max_depth <= 32. */
typedef struct hasty_pm_stats {
  int32_t iterations;          /* iterations rendered */
  int64_t photons_emitted;     /* last iteration */
  int64_t photons_stored;      /* last iteration */
  float cell_size;             /* hash-cell size of the last iteration */
  double device_ms;            /* photon tracing, map build and gather kernels, all iterations */
  double host_ms;              /* wall time minus device_ms, all iterations */
  uint64_t media_overflow;     /* medium-stack pushes beyond 4 (dropped) */
  uint64_t trial_cap;          /* rejection loops that hit their bound */
  double photon_ms;            /* of device_ms: photon emission and tracing */
  double gather_ms;            /* of device_ms: per-pixel gather */
  double cell_ms;              /* host time of the hash-cell size (computeCellSize), run while photons are traced */
  double map_ms;               /* of device_ms: photon-map build (order, sort by cell, cell table) */
} hasty_pm_stats;

/* Renders `iterations` more progressive iterations (synchronous). */
int hasty_pm_render(hasty_job* job, int iterations);
/* Restarts from the initial radii and empty statistics at the next render. */
int hasty_pm_reset(hasty_job* job);
/* Current estimate (w*h*3 floats): colour (x 2^exposure), normal or albedo
 * of the last iteration, as the reference's thread image buffers. */
int hasty_pm_read(hasty_job* job, int aov, float* host_rgb, size_t w, size_t h);
/* Per-pixel gather radii after the last iteration (w*h floats). */
int hasty_pm_read_radii(hasty_job* job, float* host, size_t w, size_t h);
int hasty_pm_stats_get(hasty_job* job, hasty_pm_stats* stats);
/* Photon map of the last iteration, for tests: photons in map order
 * (position xyz[3n], emission index, index among the photons that emission
 * stored) and the cell table cells[5 * n_cells] = (x, y, z, first photon,
 * count). With null buffers only *n_photons, *n_cells and *cell are set. */
int hasty_debug_pm_map(hasty_job* job, float* xyz, uint32_t* emission, uint32_t* index, int32_t* cells,
                       int64_t* n_photons, int64_t* n_cells, float* cell);

/* ---- Batching: many jobs in one multi-job wavefront ----------------------
 * Two modes.
 * HASTY_BATCH_PACKED (default): the jobs' passes are packed, in job order,
 * into batches of up to paths_in_flight camera samples (chunks of
 * consecutive passes of several jobs side by side); each batch runs the
 * single-job path's wavefront kernels with the chunk table as a kernel
 * parameter, on one of `lanes` render lanes (streams) that alternate, so one
 * batch's tracing overlaps another's shading. Accumulation adds each pass to
 * the job's FP64 sums in pass order, so a job's result is bit-identical to
 * hasty_job_render_passes of the same passes, alone or in any mix.
 * HASTY_BATCH_REGEN: path slots are shared by all jobs and refilled with new
 * camera samples as paths finish (regeneration); one CUDA graph launch whose
 * conditional while-node repeats regenerate/trace/shade on the device runs
 * the whole batch. Two such engines, each with half the pool and its own
 * stream, take alternate passes of every job so that one's tracing overlaps
 * the other's shading. Each job's samples are accumulated in int64 fixed
 * point (2^-32), which is order-independent: a job's result is bit-identical
 * alone or in any mix, on one engine or two, and equal to the FP64 sums to
 * 2^-32 per sample.
 * No counterpart in the reference (its jobs run one at a time). */
#define HASTY_BATCH_PACKED 0
#define HASTY_BATCH_REGEN 1

typedef struct hasty_batch_config {
  int64_t paths_in_flight;     /* packed: path slots per lane, 0 = 16M; regen: the shared pool, 0 = 4M */
  float regen_fraction;        /* regen: refill when live paths < fraction * pool; 0 = 0.9, >= 1 every iteration */
  int32_t max_iterations;      /* regen: device-side loop bound; 0 = 50M */
  int32_t mode;                /* HASTY_BATCH_PACKED or HASTY_BATCH_REGEN */
  int32_t lanes;               /* packed: render lanes (batches in flight), 1..4; 0 = 2 */
  int32_t resolve_threads;     /* packed: block size of the resolve kernel, 128 or 256; 0 = 256 */
  int32_t sample_threads;      /* packed: block size of the sample kernel, 256 or 512; 0 = 512 */
  int32_t trace_blocks_per_sm; /* packed: closest-hit blocks per SM while batches overlap; 0 = 5 */
  int32_t pad;
} hasty_batch_config;

typedef struct hasty_batch_stats {
  double device_ms;            /* device time of the batch (CUDA events) */
  double wall_ms;              /* host wall time including engine set-up */
  uint64_t samples;            /* camera samples rendered */
  uint64_t rays;
  uint64_t shaded;
  uint64_t nan_samples;
  uint64_t saturated;          /* regen: samples clamped to +/-2^30 in fixed point */
  uint64_t iterations;         /* regen: engine iterations (the longer engine); packed: batches */
  int64_t paths_in_flight;     /* path slots of all lanes / both engines together */
  int64_t engine_bytes;        /* device memory of the lanes or engines (path state, fixed-point sums) */
  uint64_t kernel_launches;    /* packed: kernels launched */
  uint64_t media_overflow;     /* medium-stack pushes dropped (beyond 20 nested media; regen: beyond 4) */
} hasty_batch_stats;

/* Renders passes[i] further passes of jobs[i] (all from ctx) in one run and
 * adds the results to each job's accumulators, as hasty_job_render_passes
 * would; synchronous. */
int hasty_batch_render(hasty_ctx* ctx, hasty_job** jobs, const int32_t* passes, size_t n_jobs,
                       const hasty_batch_config* cfg, hasty_batch_stats* stats);

/* ---- Serving: a request loop over packed multi-job batches ----------------
 * Requests (a renderJob.json, a pass count, a seed) are admitted while job
 * slots and the device-memory budget allow: scene + BVH + textures of each
 * resident scene, 72 B per pixel of FP64 sums per resident request, plus the
 * render lanes' path state. Scenes are cached by scene file and shared by
 * the requests that use them; a scene no request uses is evicted when room is
 * needed. Loader threads parse scenes and build BVHs on the host while the
 * GPU renders. The passes of the resident requests are packed into batches
 * (as hasty_batch_render's packed mode) that run on `lanes` render lanes, a
 * new batch being formed whenever a lane frees up, so requests that arrive
 * while others render join the next batch. Each batch takes at most
 * quantum_samples camera samples of one request; requests are visited
 * round-robin (HASTY_SERVE_ROUND_ROBIN) or by fewest samples left
 * (HASTY_SERVE_SHORTEST_FIRST). A request's sums are added pass by pass in
 * FP64, so its result is bit-identical to hasty_job_render_passes (and to
 * hasty_batch_render) of the same job, seed and pass count, alone or in any
 * mix. The server's functions are internally synchronised (any host thread).
 * No counterpart in the reference (its viewer renders one job per process). */
typedef struct hasty_server hasty_server;

#define HASTY_SERVE_ROUND_ROBIN 0
#define HASTY_SERVE_SHORTEST_FIRST 1

typedef struct hasty_server_config {
  int64_t paths_in_flight;     /* path slots per render lane; 0 = 16M (raised to the largest frame) */
  int32_t lanes;               /* render lanes (batches in flight), 1..4; 0 = 2 */
  int32_t max_resident_jobs;   /* requests rendering at once; 0 = 32 */
  int32_t max_resident_scenes; /* scenes kept on the device; 0 = 32 */
  int32_t loader_threads;      /* 0 = 2 */
  int64_t memory_budget;       /* device bytes; 0 = 120 GB */
  int64_t quantum_samples;     /* camera samples of one request per batch at most; 0 = paths_in_flight / 4 */
  int32_t policy;              /* HASTY_SERVE_ROUND_ROBIN (0) or HASTY_SERVE_SHORTEST_FIRST */
  int32_t resolve_threads;     /* block shapes, as hasty_batch_config; 0 = defaults */
  int32_t sample_threads;
  int32_t trace_blocks_per_sm;
} hasty_server_config;

typedef struct hasty_server_result {
  int64_t id;
  int32_t status;              /* HASTY_OK, or the code the request failed with */
  int32_t width, height;
  int32_t passes;
  uint64_t samples;            /* camera samples rendered (passes * width * height) */
  double submit_ms, admit_ms, finish_ms;   /* since hasty_server_start */
  double latency_ms;           /* finish_ms - submit_ms */
  char error[160];             /* message when status != HASTY_OK */
} hasty_server_result;

typedef struct hasty_server_stats {
  uint64_t submitted, admitted, completed, failed;
  uint64_t samples;            /* camera samples of completed requests */
  uint64_t rays, shaded;
  uint64_t batches;            /* packed batches launched */
  uint64_t kernel_launches;
  double device_ms;            /* time the GPU had a batch in flight (CUDA events; overlapping batches once) */
  double uptime_ms;
  int64_t resident_bytes;      /* render lanes + scenes + resident requests */
  int64_t peak_resident_bytes;
  int64_t engine_bytes;        /* render lanes (path state) */
  int32_t resident_jobs, resident_scenes, pending;
} hasty_server_stats;

int hasty_server_start(hasty_ctx* ctx, const hasty_server_config* cfg, hasty_server** out);
/* passes <= 0: the job file's num_samples; seed NULL: the job file's seed. */
int hasty_server_submit(hasty_server* srv, const char* render_job_path, int32_t passes, const uint64_t* seed,
                        int64_t* id);
/* Up to max finished requests not returned before; waits up to wait_ms for
 * the first one. */
int hasty_server_poll(hasty_server* srv, hasty_server_result* out, size_t max, size_t* n, int32_t wait_ms);
/* Estimate of a finished request (as hasty_job_read) or its raw FP64 sums
 * (as hasty_job_read_sums); valid until hasty_server_release. */
int hasty_server_read(hasty_server* srv, int64_t id, int aov, float* host_rgb, size_t w, size_t h);
int hasty_server_read_sums(hasty_server* srv, int64_t id, int aov, double* host_rgb, size_t w, size_t h);
int hasty_server_release(hasty_server* srv, int64_t id);
int hasty_server_stats_get(hasty_server* srv, hasty_server_stats* out);
/* Waits until every submitted request has finished (HASTY_ERR_STOPPED on timeout). */
int hasty_server_wait_idle(hasty_server* srv, int32_t timeout_ms);
/* Stops the loop: requests not finished fail with HASTY_ERR_STOPPED; frees everything. */
int hasty_server_stop(hasty_server* srv);

/* ---- One pass without device allocation ------------------------------------
 * Renders camera-sample pass `pass` of the job (seed and settings as loaded)
 * into d_color, a caller-owned DEVICE buffer of w*h*3 doubles (row-major RGB
 * radiance of that one sample per pixel, before exposure), which it
 * overwrites. Asynchronous on the job's stream (hasty_job_sync waits). Leaves
 * the job's accumulators, pass counter and statistics untouched.
 * For callers that may not allocate device memory while rendering: the call
 * makes no cudaMalloc/cudaFree and uses one fixed 8 MiB static device array
 * as scratch, so frames above 16384 pixels (e.g. 128 x 128) are rejected
 * with HASTY_ERR_ARG. The first call on each device looks up that array's
 * address; make it before any stream capture begins; that address stays
 * cached for the process, so do not call this again after cudaDeviceReset.
 * All calls share the array: calls whose GPU work overlaps (other streams,
 * other threads) race. Each job renders on its own stream and the call is
 * asynchronous, so calls on two different jobs overlap unless the first
 * job is synced (hasty_job_sync) before the second call.
 * No counterpart in the reference (it renders through its own buffers). */
int hasty_job_render_pass_static(hasty_job* job, int pass, double* d_color);
/* Bounds-checked build only (python -m hastyrenderer_gb300.build
 * --debug-bounds, which writes lib/bounds/libhasty_gb300.so): the device
 * kernels check the indices they read through (queue entries, ray ids, BVH
 * nodes and leaf triangles, hit triangles, materials, textures, light
 * triangles, medium-stack blocks) and on a bad one skip the access and set
 * a bit; this returns the bits set since the last call (HASTY_BOUNDS_*) and
 * clears them. The regular build returns HASTY_ERR_MISSING. No counterpart
 * in the reference. */
#define HASTY_BOUNDS_QUEUE 1u
#define HASTY_BOUNDS_NODE 2u
#define HASTY_BOUNDS_LEAF_TRI 4u
#define HASTY_BOUNDS_TRI 8u
#define HASTY_BOUNDS_MATERIAL 16u
#define HASTY_BOUNDS_TEXTURE 32u
#define HASTY_BOUNDS_LIGHT 64u
#define HASTY_BOUNDS_MEDIA 128u
int hasty_debug_bounds_status(uint32_t* flags);
/* Test hook (no device needed): the static scratch's pixel limit, the bytes a
 * frame of that many pixels carves from it, and its size. */
int hasty_debug_static_scratch(int64_t* max_pixels, int64_t* bytes_needed, int64_t* capacity);
/* Test hook (no device needed): the packed-batch plan hasty_batch_render
 * and the server follow, for n_jobs jobs of npix[i] pixels, passes[i]
 * passes and kernel class cls[i] (0 wavefront with the persistent
 * closest-hit kernel, 1 wavefront with one ray per thread, 2 path kernel),
 * `slots` path slots per batch and at most job_samples camera samples of one
 * job per batch (0: no limit). Writes one (batch, job, first pass, passes)
 * quadruple of int32 per chunk, in launch order, up to max_chunks, and the
 * number of chunks planned into n_out. */
int hasty_debug_pack(const int32_t* npix, const int32_t* passes, const int32_t* cls, size_t n_jobs, int64_t slots,
                     int64_t job_samples, int32_t* out, size_t max_chunks, size_t* n_out);

/* Closest hits of n rays given as n x 6 host floats (origin, direction):
 * global triangle index (-1 miss), t, u, v. */
/* Parses an OBJ file with `chunks` parse chunks (0: automatic), no device
 * needed, for tests: a digest of the triangles (corner indices, materials,
 * smoothing groups, shape boundaries) and their counts. */
int hasty_debug_obj_digest(const char* path, int chunks, uint64_t* digest, int64_t* n_tris, int64_t* n_shapes);
int hasty_debug_intersect(hasty_job* job, const float* rays, size_t n, int32_t* tri, float* t, float* u, float* v);
/* The same closest-hit traversal run on the CPU (no device needed): loads the
 * job on the host, builds the BVH (kind 0 binary, 1 compressed 8-wide) and
 * answers n rays. info (may be NULL): triangles, nodes, tree depth. */
int hasty_debug_host_trace(const char* render_job_path, int kind, const float* rays, size_t n, int32_t* tri, float* t,
                           float* u, float* v, int64_t* info);
/* Builds the BVH tree of a job on `device`, writes the compressed 8-wide
 * layout on the device and on the host from that same tree, and reports
 * whether the two are byte-identical (identical = 1). info (8 values, may be
 * NULL): device and host node counts, first differing node word (-1 none),
 * device and host depth, triangles equal, order equal, two device builds
 * equal. */
int hasty_debug_wide_emit_check(int device, const char* render_job_path, int64_t* info, int32_t* identical);
/* Triangle index -> (OBJ shape = Embree geomID, face = primID). */
int hasty_debug_tri_ids(hasty_job* job, int32_t* geom, int32_t* prim, size_t n);
/* BSDF known-answer evaluation on the device. which: 0 sample, 1 evaluate, 2 pdf.
 * in: n_cases x 33 floats; replay: n_cases x n_replay u32 values, case c draws
 * replay[c*n_replay ...] in order; out: n_cases x 12 floats. */
int hasty_debug_bsdf(int which, const float* in, size_t n_cases, const uint32_t* replay, size_t n_replay, float* out);

#ifdef __cplusplus
}
#endif

#endif /* HASTY_GPU_H */
