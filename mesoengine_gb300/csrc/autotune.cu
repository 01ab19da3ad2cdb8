// autotune.cu -- grid search of the launch knobs on synthetic inputs.
//
// The reference fixes its batching by hand in FVoxelSceneConfig
// (ChunkTaskPerCore = 8, MaxUnsyncedLoadChunkCount = 256,
// Runtimes/Voxel/VoxelSceneConfig.h:35-37).  Here the knobs are the ray tile
// width (lanes of a warp along x) and warps per CTA of the raymarch launch,
// and the chunks taken per queue ticket of the persistent mesher; each
// candidate is timed with CUDA events and the fastest is applied to the
// context and written as flat JSON that meso_config.tuning_path reads back.
#include <cmath>
#include <cstdio>
#include <cstring>
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

extern "C" meso_status meso_autotune(meso_ctx* ctx, const char* path) {
  if (!ctx) return fail(MESO_ERR_INVALID_ARG, "autotune: null ctx");
  cudaStream_t st = ctx->stream;
  const Tuning saved = ctx->tuning;
  // ---- raymarch: 512^3 terrain, 1280x720 primary + shadow
  meso_terrain t = {512, 512, 512, 11, 256, 6, 28.0f, 128.0f, 48, 0.7f};
  meso_scene* scene = nullptr;
  MESO_TRY(scene_create_terrain(ctx, &t, 0, &scene));
  const float o[3] = {-150.0f, -100.0f, 400.0f}, tg[3] = {256.0f, 256.0f, 256.0f};
  const meso_camera cam = look_at(o, tg, 1280, 720);
  const float light[3] = {0.30304575f, 0.50507629f, 0.80812204f};  // normalize(0.3, 0.5, 0.8)
  meso_hit* d_hits = nullptr;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  meso_status rc = MESO_OK;
  cudaError_t e = cudaMalloc(&d_hits, sizeof(meso_hit) * 1280 * 720);
  if (e != cudaSuccess) rc = cuda_fail(e, "autotune: hit buffer");
  const meso_scene* sc = scene;
  float best_ray = 1e30f;
  Tuning best = saved;
  const uint32_t tws[4] = {4, 8, 16, 32}, wpcs[3] = {1, 2, 4};  // the kernel allows at most 128 threads per CTA
  for (uint32_t tw : tws) {
    for (uint32_t wpc : wpcs) {
      if (rc != MESO_OK) break;
      ctx->tuning.ray_tile_w = tw;
      ctx->tuning.ray_warps_per_cta = wpc;
      for (int w = 0; w < 2; w++) launch_raymarch(ctx, &sc, &cam, 1, light, MESO_RAY_SHADOW, d_hits, st, nullptr, 0);
      cudaEventRecord(a, st);
      for (int k = 0; k < 5; k++) rc = launch_raymarch(ctx, &sc, &cam, 1, light, MESO_RAY_SHADOW, d_hits, st, nullptr, 0);
      cudaEventRecord(b, st);
      cudaEventSynchronize(b);
      float ms = 0;
      cudaEventElapsedTime(&ms, a, b);
      if (rc == MESO_OK && ms < best_ray) {
        best_ray = ms;
        best.ray_tile_w = tw;
        best.ray_warps_per_cta = wpc;
      }
    }
  }
  cudaFree(d_hits);
  scene_release(ctx, scene);
  // ---- mesher: 1024 generated standalone chunks
  const uint32_t n = 1024;
  uint16_t* d_chunks = nullptr;
  uint64_t* d_quads = nullptr;
  uint64_t* d_count = nullptr;
  const uint64_t cap = (uint64_t)n * 16384;
  float best_mesh = 1e30f;
  if (rc == MESO_OK) {
    e = cudaMalloc(&d_chunks, (size_t)n * 65536);
    if (e == cudaSuccess) e = cudaMalloc(&d_quads, cap * 8);
    if (e == cudaSuccess) e = cudaMalloc(&d_count, 8);
    if (e != cudaSuccess) rc = cuda_fail(e, "autotune: mesh buffers");
  }
  if (rc == MESO_OK) rc = generate_chunks_u16(ctx, n, 1, d_chunks, nullptr, st);
  ctx->tuning = best;
  const uint32_t tickets[3] = {1, 2, 4};
  for (uint32_t per : tickets) {
    if (rc != MESO_OK) break;
    ctx->tuning.mesh_chunks_per_ticket = per;
    meso_mesh_source src;
    memset(&src, 0, sizeof(src));
    src.kind = MESO_SRC_CHUNKS_U16;
    src.d_data = d_chunks;
    meso_mesh_output out = {d_quads, cap, d_count, nullptr};
    for (int w = 0; w < 2; w++) launch_mesh(ctx, &src, nullptr, n, &out, st, false);
    cudaEventRecord(a, st);
    for (int k = 0; k < 5; k++) rc = launch_mesh(ctx, &src, nullptr, n, &out, st, false);
    cudaEventRecord(b, st);
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    if (rc == MESO_OK && ms < best_mesh) {
      best_mesh = ms;
      best.mesh_chunks_per_ticket = per;
    }
  }
  cudaFree(d_chunks);
  cudaFree(d_quads);
  cudaFree(d_count);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc != MESO_OK) {
    ctx->tuning = saved;
    return rc;
  }
  best.mesh_ctas_per_sm = 0;  // the default: two 16-warp CTAs per SM, what registers and shared memory allow
  ctx->tuning = best;
  if (path && *path) {
    FILE* f = fopen(path, "w");
    if (!f) return fail(MESO_ERR_INVALID_ARG, std::string("autotune: cannot write ") + path);
    fprintf(f,
            "{\"mesh_ctas_per_sm\": %u, \"mesh_chunks_per_ticket\": %u, \"ray_tile_w\": %u, "
            "\"ray_warps_per_cta\": %u, \"ray_ms_1280x720\": %.4f, \"mesh_ms_1024_chunks\": %.4f, \"sm_count\": %d}\n",
            best.mesh_ctas_per_sm, best.mesh_chunks_per_ticket, best.ray_tile_w, best.ray_warps_per_cta,
            best_ray / 5.0f, best_mesh / 5.0f, ctx->sm_count);
    fclose(f);
  }
  return MESO_OK;
}
