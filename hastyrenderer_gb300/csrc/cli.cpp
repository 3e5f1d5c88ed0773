// hasty_gpu_render <renderJob.json> <outputDirectory>
// Headless counterpart of the reference's PathTracingViewer
// (apps/PathTracingViewer.cpp:17-175): same arguments, renders
// settings.num_samples passes, writes output.exr, outputNormal.exr and
// outputAlbedo.exr. Exit codes: 1 bad arguments or output directory, 2 load
// failure, 5 save failure, 3 CUDA failure (the reference uses 3/4 for its SDL
// window, which does not exist here). The denoised output is not produced.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <sys/stat.h>

#include "hasty_gpu.h"

int main(int argc, char** argv) {
  if (argc != 3) {
    std::printf("unexpected number of arguments: %d expecting 3, usage <binary> <renderJobFile> <outputDirectory> \n", argc);
    return 1;
  }
  struct stat sb;
  if (stat(argv[2], &sb) != 0 || !S_ISDIR(sb.st_mode)) {
    std::printf("error given output path %s is not a directory \n", argv[2]);
    return 1;
  }
  char err[1024];
  hasty_ctx* ctx = nullptr;
  if (hasty_ctx_create(0, 0, &ctx) != HASTY_OK) { hasty_last_error(err, sizeof err); std::printf("cuda error: %s\n", err); return 3; }
  hasty_job* job = nullptr;
  if (hasty_job_load(ctx, argv[1], &job) != HASTY_OK) {
    hasty_last_error(err, sizeof err);
    std::printf("exception: %s\n", err);
    hasty_ctx_destroy(ctx);
    return 2;
  }
  hasty_job_info info;
  hasty_job_info_get(job, &info);
  // HASTY_WRITE_EVERY=k (> 0): the outputs are also written every k passes
  // while rendering continues, as the reference's window shows the estimate
  // during the render (apps/PathTracingViewer.cpp:88-139).
  int every = 0;
  if (const char* e = std::getenv("HASTY_WRITE_EVERY")) every = std::atoi(e);
  auto t0 = std::chrono::steady_clock::now();
  int rc = HASTY_OK;
  if (every > 0) {
    int wrc = HASTY_OK;
    for (int done = 0; rc == HASTY_OK && wrc == HASTY_OK && done < info.num_samples; done += every) {
      rc = hasty_job_render_passes(job, std::min(every, info.num_samples - done));
      if (rc == HASTY_OK) wrc = hasty_job_write_outputs_async(job, argv[2], 0);
    }
    if (wrc == HASTY_OK) wrc = hasty_job_outputs_wait(job);
    if (rc == HASTY_OK && wrc != HASTY_OK) {
      hasty_last_error(err, sizeof err);
      std::printf("exception: %s\n", err);
      hasty_job_destroy(job); hasty_ctx_destroy(ctx);
      return 5;
    }
  } else {
    rc = hasty_job_render_passes(job, info.num_samples);
  }
  if (rc == HASTY_OK) rc = hasty_job_sync(job);
  double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (rc != HASTY_OK) {
    hasty_last_error(err, sizeof err); std::printf("render failed: %s\n", err);
    hasty_job_destroy(job); hasty_ctx_destroy(ctx);
    return 3;
  }
  std::printf("%d samples per pixel, %dx%d, %.3f s, %.1f Msamples/s\n", info.num_samples, info.width, info.height, s,
              double(info.num_samples) * info.width * info.height / s * 1e-6);
  std::printf(" writing raw files to disk \n");
  if (hasty_job_write_outputs(job, argv[2], 0) != HASTY_OK) {
    hasty_last_error(err, sizeof err);
    std::printf("exception: %s\n", err);
    hasty_job_destroy(job); hasty_ctx_destroy(ctx);
    return 5;
  }
  hasty_job_destroy(job);
  hasty_ctx_destroy(ctx);
  return 0;
}
