// autotune.cu -- grid search of the launch knobs on synthetic inputs.
//
// The reference fixes its batching by hand in FVoxelSceneConfig
// (ChunkTaskPerCore = 8, MaxUnsyncedLoadChunkCount = 256,
// Runtimes/Voxel/VoxelSceneConfig.h:35-37).  Here the knobs are the ray tile
// width (lanes of a warp along x) and warps per CTA of the raymarch launch
// (its tile shape), and the persistent mesher's CTAs per SM (bricks in flight
// per SM: a CTA meshes one 32^3 chunk of 64 bricks at a time) and chunks
// taken per queue ticket (its queue granularity); each
// candidate is timed with CUDA events and the fastest is applied to the
// context and written as flat JSON that meso_config.tuning_path reads back.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "meso_internal.h"

namespace meso {
meso_status scene_create_terrain(meso_ctx*, const meso_terrain*, uint64_t, meso_scene**);
meso_status generate_chunks_u16(meso_ctx*, uint32_t, uint32_t, uint16_t*, uint32_t*, cudaStream_t);
}  // namespace meso

namespace {

meso_camera look_at(const float o[3], const float tgt[3], uint32_t w, uint32_t h) {
  meso_camera c;
  memset(&c, 0, sizeof(c));
  float f[3] = {tgt[0] - o[0], tgt[1] - o[1], tgt[2] - o[2]};
  float n = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
  for (float& v : f) v /= n;
  float r[3] = {f[1], -f[0], 0.0f};  // f x (0,0,1)
  n = std::sqrt(r[0] * r[0] + r[1] * r[1]);
  for (float& v : r) v /= n;
  const float u[3] = {r[1] * f[2] - r[2] * f[1], r[2] * f[0] - r[0] * f[2], r[0] * f[1] - r[1] * f[0]};
  for (int a = 0; a < 3; a++) {
    const int ch = (int)std::floor(o[a] / 32.0f);
    c.origin_chunk[a] = ch;
    c.origin_frac[a] = o[a] - 32.0f * (float)ch;
    c.forward[a] = f[a];
    c.right[a] = r[a];
    c.up[a] = u[a];
  }
  c.tan_half_fov_y = std::tan(30.0f * 3.14159265f / 180.0f);
  c.width = w;
  c.height = h;
  return c;
}

}  // namespace

using namespace meso;

namespace {

// Times `reps` calls of fn() (after two untimed warm-up calls) on stream st
// with the events a and b; any failing status ends the measurement.
template <typename F>
meso_status time_calls(cudaStream_t st, cudaEvent_t a, cudaEvent_t b, int reps, F fn, float* ms) {
  for (int w = 0; w < 2; w++) MESO_TRY(fn());
  MESO_CUDA_TRY(cudaEventRecord(a, st));
  for (int k = 0; k < reps; k++) MESO_TRY(fn());
  MESO_CUDA_TRY(cudaEventRecord(b, st));
  MESO_CUDA_TRY(cudaEventSynchronize(b));
  MESO_CUDA_TRY(cudaEventElapsedTime(ms, a, b));
  return MESO_OK;
}

struct TuneScratch {
  meso_ctx* ctx = nullptr;
  meso_scene* scene = nullptr;
  meso_hit* d_hits = nullptr;
  uint16_t* d_chunks = nullptr;
  uint64_t* d_quads = nullptr;
  uint64_t* d_count = nullptr;
  cudaEvent_t a = nullptr, b = nullptr;
  ~TuneScratch() {
    if (ctx) cudaStreamSynchronize(ctx->stream);
    if (scene) scene_release(ctx, scene);
    cudaFree(d_hits);  // cudaFree(nullptr) is a no-op
    cudaFree(d_chunks);
    cudaFree(d_quads);
    cudaFree(d_count);
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
  }
};

meso_status autotune_search(meso_ctx* ctx, Tuning& best, float& best_ray, float& best_mesh) {
  cudaStream_t st = ctx->stream;
  TuneScratch S;
  S.ctx = ctx;
  MESO_CUDA_TRY(cudaEventCreate(&S.a));
  MESO_CUDA_TRY(cudaEventCreate(&S.b));
  // ---- raymarch tile shape: 512^3 terrain, 1280x720 primary + shadow
  meso_terrain t = {512, 512, 512, 11, 256, 6, 28.0f, 128.0f, 48, 0.7f};
  MESO_TRY(scene_create_terrain(ctx, &t, 0, &S.scene));
  const float o[3] = {-150.0f, -100.0f, 400.0f}, tg[3] = {256.0f, 256.0f, 256.0f};
  const meso_camera cam = look_at(o, tg, 1280, 720);
  const float light[3] = {0.30304575f, 0.50507629f, 0.80812204f};  // normalize(0.3, 0.5, 0.8)
  MESO_CUDA_TRY(cudaMalloc(&S.d_hits, sizeof(meso_hit) * 1280 * 720));
  const meso_scene* sc = S.scene;
  best_ray = 1e30f;
  const uint32_t tws[4] = {4, 8, 16, 32}, wpcs[3] = {1, 2, 4};  // the kernel allows at most 128 threads per CTA
  for (uint32_t tw : tws) {
    for (uint32_t wpc : wpcs) {
      ctx->tuning.ray_tile_w = tw;
      ctx->tuning.ray_warps_per_cta = wpc;
      float ms = 0.0f;
      MESO_TRY(time_calls(st, S.a, S.b, 5, [&] {
        return launch_raymarch(ctx, &sc, &cam, 1, light, MESO_RAY_SHADOW, S.d_hits, st, nullptr, 0);
      }, &ms));
      if (ms < best_ray) {
        best_ray = ms;
        best.ray_tile_w = tw;
        best.ray_warps_per_cta = wpc;
      }
    }
  }
  // ---- mesher block residency and queue granularity: 1024 generated
  // standalone chunks; a CTA meshes one 32^3 chunk (64 bricks) at a time, so
  // CTAs per SM x 64 is the bricks in flight per SM
  const uint32_t n = 1024;
  const uint64_t cap = (uint64_t)n * 16384;
  MESO_CUDA_TRY(cudaMalloc(&S.d_chunks, (size_t)n * 65536));
  MESO_CUDA_TRY(cudaMalloc(&S.d_quads, cap * 8));
  MESO_CUDA_TRY(cudaMalloc(&S.d_count, 8));
  MESO_TRY(generate_chunks_u16(ctx, n, 1, S.d_chunks, nullptr, st));
  meso_mesh_source src;
  memset(&src, 0, sizeof(src));
  src.kind = MESO_SRC_CHUNKS_U16;
  src.d_data = S.d_chunks;
  const meso_mesh_output out = {S.d_quads, cap, S.d_count, nullptr};
  best_mesh = 1e30f;
  const uint32_t ctas[2] = {1, 2}, tickets[3] = {1, 2, 4};
  for (uint32_t c : ctas) {
    for (uint32_t per : tickets) {
      ctx->tuning.mesh_ctas_per_sm = c;
      ctx->tuning.mesh_chunks_per_ticket = per;
      float ms = 0.0f;
      MESO_TRY(time_calls(st, S.a, S.b, 5, [&] { return launch_mesh(ctx, &src, nullptr, n, &out, st, false); }, &ms));
      if (ms < best_mesh) {
        best_mesh = ms;
        best.mesh_ctas_per_sm = c;
        best.mesh_chunks_per_ticket = per;
      }
    }
  }
  MESO_CUDA_TRY(cudaStreamSynchronize(st));
  uint32_t err = 0;
  MESO_CUDA_TRY(cudaMemcpy(&err, ctx->d_scratch + 1, 4, cudaMemcpyDeviceToHost));
  if (err) return fail(MESO_ERR_CUDA, "autotune: a timed launch raised the device error flag");
  return MESO_OK;
}

}  // namespace

extern "C" meso_status meso_autotune(meso_ctx* ctx, const char* path) {
  if (!ctx) return fail(MESO_ERR_INVALID_ARG, "autotune: null ctx");
  const Tuning saved = ctx->tuning;
  Tuning best = saved;
  float best_ray = 0.0f, best_mesh = 0.0f;
  const meso_status rc = autotune_search(ctx, best, best_ray, best_mesh);
  if (rc != MESO_OK) {
    ctx->tuning = saved;
    return rc;
  }
  ctx->tuning = best;
  if (path && *path) {
    FILE* f = fopen(path, "w");
    if (!f) return fail(MESO_ERR_INVALID_ARG, std::string("autotune: cannot write ") + path);
    const int w = fprintf(f,
                          "{\"mesh_ctas_per_sm\": %u, \"mesh_chunks_per_ticket\": %u, \"ray_tile_w\": %u, "
                          "\"ray_warps_per_cta\": %u, \"ray_ms_1280x720\": %.4f, \"mesh_ms_1024_chunks\": %.4f, "
                          "\"sm_count\": %d}\n",
                          best.mesh_ctas_per_sm, best.mesh_chunks_per_ticket, best.ray_tile_w, best.ray_warps_per_cta,
                          best_ray / 5.0f, best_mesh / 5.0f, ctx->sm_count);
    if (fclose(f) != 0 || w < 0) return fail(MESO_ERR_INVALID_ARG, std::string("autotune: cannot write ") + path);
  }
  return MESO_OK;
}
