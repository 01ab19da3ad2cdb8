// capi.cu -- the extern "C" boundary of mesoengine_gb300 (declared in
// include/meso.h): context, device memory/stream/event helpers, scenes,
// meshing and raymarching entry points.  No exception crosses this layer;
// every failure becomes a meso_status plus a per-thread message.
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "meso_internal.h"

namespace meso {

static thread_local std::string g_err;

void set_error(const std::string& msg) { g_err = msg; }

meso_status fail(meso_status s, const std::string& msg) {
  g_err = msg;
  return s;
}

meso_status cuda_fail(cudaError_t e, const char* what) {
  g_err = std::string(what) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? MESO_ERR_OOM : MESO_ERR_CUDA;
}

// defined in scene.cu
meso_status scene_create_terrain(meso_ctx*, const meso_terrain*, uint64_t, meso_scene**);
meso_status scene_create_dense(meso_ctx*, const uint16_t*, int32_t, int32_t, int32_t, uint64_t, meso_scene**);
meso_status scene_create_grid(meso_ctx*, int32_t, const void*, int32_t, int32_t, int32_t, uint64_t, meso_scene**);
meso_status scene_count_solid(meso_ctx*, const meso_scene*, uint64_t*);
meso_status generate_dense_u8(meso_ctx*, int32_t, int32_t, int32_t, uint32_t, uint8_t*, cudaStream_t);
meso_status generate_chunks_u16(meso_ctx*, uint32_t, uint32_t, uint16_t*, uint32_t*, cudaStream_t);
meso_status edit_spheres(meso_ctx*, meso_scene*, const meso_sphere_edit*, uint32_t, uint32_t*, uint32_t, uint32_t*,
                         cudaStream_t);

// Minimal reader for the tuning JSON written by meso_autotune: flat
// {"key": number, ...}.
static void load_tuning(const char* path, Tuning& t) {
  if (!path || !*path) return;
  std::ifstream f(path);
  if (!f) return;
  std::stringstream ss;
  ss << f.rdbuf();
  const std::string s = ss.str();
  auto num = [&](const char* key, uint32_t& dst) {
    const std::string k = std::string("\"") + key + "\"";
    size_t p = s.find(k);
    if (p == std::string::npos) return;
    p = s.find(':', p);
    if (p == std::string::npos) return;
    long v = strtol(s.c_str() + p + 1, nullptr, 10);
    if (v > 0 && v < 1 << 20) dst = (uint32_t)v;
  };
  num("mesh_ctas_per_sm", t.mesh_ctas_per_sm);
  num("mesh_chunks_per_ticket", t.mesh_chunks_per_ticket);
  num("ray_tile_w", t.ray_tile_w);
  num("ray_warps_per_cta", t.ray_warps_per_cta);
}

}  // namespace meso

using namespace meso;

namespace {
// An mbarrier that nothing arrives on: its phase 0 never completes, so the
// bounded wait must give up; the kernel flags it as every copy wait does.
__global__ void bounded_wait_probe_kernel(uint64_t limit_ns, uint32_t* err) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    meso::dev::mbar_init(&bar, 1);
    meso::dev::fence_proxy_async_smem();
  }
  __syncthreads();
  const bool ok = meso::dev::mbar_wait_bounded(&bar, 0, limit_ns);
  if (!ok && threadIdx.x == 0) atomicOr(err, meso::ERR_TIMEOUT);
}

// Reads an L2-resident buffer `passes` times with 16-byte cache-global loads
// (L1 bypassed); the XOR of every word keeps the loads from being dropped.
__global__ void l2_read_kernel(const uint4* __restrict__ buf, size_t n16, uint32_t passes, uint32_t* sink) {
  uint32_t acc = 0;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (uint32_t k = 0; k < passes; k++) {
#pragma unroll 4
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += stride) {
      const uint4 v = __ldcg(buf + i);
      acc ^= v.x ^ v.y ^ v.z ^ v.w;
    }
  }
  if (acc == 0x9E3779B9u) atomicAdd(sink, 1u);
}
}  // namespace

extern "C" {

const char* meso_last_error_string(void) { return g_err.c_str(); }

const char* meso_status_string(meso_status s) {
  switch (s) {
    case MESO_OK: return "ok";
    case MESO_ERR_INVALID_ARG: return "invalid argument";
    case MESO_ERR_OOM: return "out of memory";
    case MESO_ERR_OVER_BUDGET: return "over HBM budget";
    case MESO_ERR_OVERFLOW: return "output overflow";
    case MESO_ERR_TIMEOUT: return "device wait timed out";
    case MESO_ERR_CUDA: return "CUDA error";
    case MESO_ERR_NOT_READY: return "not ready";
    case MESO_ERR_SHUTDOWN: return "shut down";
  }
  return "unknown";
}

meso_status meso_ctx_create(const meso_config* cfg, meso_ctx** out) {
  if (!out) return fail(MESO_ERR_INVALID_ARG, "ctx_create: null out");
  *out = nullptr;
  meso_config c;
  memset(&c, 0, sizeof(c));
  if (cfg) c = *cfg;
  if ((c.chunk_edge && c.chunk_edge != 32) || (c.brick_edge && c.brick_edge != 8))
    return fail(MESO_ERR_INVALID_ARG, "ctx_create: chunk edge must be 32 and brick edge 8");
  int n = 0;
  MESO_CUDA_TRY(cudaGetDeviceCount(&n));
  if (c.device < 0 || c.device >= n) return fail(MESO_ERR_INVALID_ARG, "ctx_create: no such device");
  MESO_CUDA_TRY(cudaSetDevice(c.device));
  cudaDeviceProp prop;
  MESO_CUDA_TRY(cudaGetDeviceProperties(&prop, c.device));
  if (prop.major < 10) return fail(MESO_ERR_CUDA, "ctx_create: needs a Blackwell (sm_10x) device");
  meso_ctx* ctx = new meso_ctx();
  ctx->device = c.device;
  ctx->sm_count = prop.multiProcessorCount;
  load_tuning(c.tuning_path, ctx->tuning);
  if (ctx->tuning.ray_warps_per_cta > 4) ctx->tuning.ray_warps_per_cta = 4;  // files from older tunings
  if (ctx->tuning.mesh_ctas_per_sm > 2) ctx->tuning.mesh_ctas_per_sm = 0;  // 0: two CTAs per SM
  if (c.mesh_ctas_per_sm) ctx->tuning.mesh_ctas_per_sm = c.mesh_ctas_per_sm;
  if (c.mesh_chunks_per_ticket) ctx->tuning.mesh_chunks_per_ticket = c.mesh_chunks_per_ticket;
  if (c.ray_tile_w) ctx->tuning.ray_tile_w = c.ray_tile_w;
  if (c.ray_warps_per_cta) ctx->tuning.ray_warps_per_cta = c.ray_warps_per_cta;
  if (32 % ctx->tuning.ray_tile_w || ctx->tuning.ray_warps_per_cta == 0 || ctx->tuning.ray_warps_per_cta > 4 ||
      ctx->tuning.mesh_ctas_per_sm > 2) {
    delete ctx;
    return fail(MESO_ERR_INVALID_ARG, "ctx_create: bad ray tile or mesher configuration");
  }
  size_t free_b = 0, total_b = 0;
  cudaMemGetInfo(&free_b, &total_b);
  ctx->budget_bytes = c.hbm_budget_bytes ? c.hbm_budget_bytes : (uint64_t)(free_b * 0.9);
  cudaError_t e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&ctx->d_scratch, 64);
  if (e == cudaSuccess) e = cudaMemset(ctx->d_scratch, 0, 64);
  if (e == cudaSuccess) e = cudaMalloc(&ctx->d_tickets, 4 * meso_ctx::kTicketRing);
  if (e == cudaSuccess) e = cudaMemset(ctx->d_tickets, 0, 4 * meso_ctx::kTicketRing);
  if (e == cudaSuccess) {
    // per-call temporaries (edit lists, view tables, staging) come from the
    // device's default stream-ordered pool; keeping up to 1 GiB of freed
    // blocks cached there lets the next call reuse them instead of mapping
    // fresh memory (which cost ~0.15 ms per sphere-edit call)
    cudaMemPool_t pool = nullptr;
    e = cudaDeviceGetDefaultMemPool(&pool, c.device);
    uint64_t keep = 1ull << 30, cur = 0;
    if (e == cudaSuccess) e = cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &cur);
    if (e == cudaSuccess && cur < keep) e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  if (e != cudaSuccess) {
    if (ctx->d_tickets) cudaFree(ctx->d_tickets);
    if (ctx->d_scratch) cudaFree(ctx->d_scratch);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return cuda_fail(e, "ctx_create");
  }
  *out = ctx;
  return MESO_OK;
}

void meso_ctx_destroy(meso_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  cudaFree(ctx->d_scratch);
  cudaFree(ctx->d_tickets);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
}

meso_status meso_sync(meso_ctx* ctx, void* stream) {
  if (!ctx) return fail(MESO_ERR_INVALID_ARG, "sync: null ctx");
  MESO_CUDA_TRY(cudaStreamSynchronize(pick_stream(ctx, stream)));
  uint32_t err = 0;
  MESO_CUDA_TRY(cudaMemcpy(&err, ctx->d_scratch + 1, 4, cudaMemcpyDeviceToHost));
  if (err) {
    cudaMemset(ctx->d_scratch + 1, 0, 4);
    if (err & ERR_TIMEOUT) return fail(MESO_ERR_TIMEOUT, "a device wait timed out");
    if (err & ERR_POOL_FULL) return fail(MESO_ERR_OOM, "brick pool exhausted during an edit");
    if (err & ERR_BAD_INPUT) return fail(MESO_ERR_INVALID_ARG, "chunk coordinate outside the source");
  }
  return MESO_OK;
}


meso_status meso_selftest_bounded_wait(meso_ctx* ctx, uint32_t limit_us) {
  if (!ctx || limit_us == 0 || limit_us > 1000000)
    return fail(MESO_ERR_INVALID_ARG, "selftest_bounded_wait: limit must be 1..1000000 us");
  bounded_wait_probe_kernel<<<1, 32, 0, ctx->stream>>>((uint64_t)limit_us * 1000u, ctx->d_scratch + 1);
  ctx->launches.fetch_add(1);
  MESO_CUDA_TRY(cudaGetLastError());
  return meso_sync(ctx, nullptr);
}

meso_status meso_measure_l2_read(meso_ctx* ctx, uint64_t bytes, uint32_t passes, double* gb_s) {
  if (!ctx || !gb_s || bytes < (16u << 10) || bytes > (64u << 20) || bytes % 16 || passes == 0 || passes > 1000)
    return fail(MESO_ERR_INVALID_ARG, "measure_l2_read: bytes must be 16 KiB .. 64 MiB (multiple of 16), passes 1..1000");
  *gb_s = 0.0;
  const cudaStream_t st = ctx->stream;
  uint4* buf = nullptr;
  MESO_CUDA_TRY(cudaMallocAsync(&buf, bytes, st));
  cudaEvent_t a = nullptr, b = nullptr;
  cudaError_t e = cudaMemsetAsync(buf, 0x5A, bytes, st);
  if (e == cudaSuccess) e = cudaEventCreate(&a);
  if (e == cudaSuccess) e = cudaEventCreate(&b);
  const dim3 grid(ctx->sm_count * 8), block(256);
  if (e == cudaSuccess) {
    l2_read_kernel<<<grid, block, 0, st>>>(buf, bytes / 16, 1, ctx->d_scratch + 2);  // brings the buffer into L2
    cudaEventRecord(a, st);
    l2_read_kernel<<<grid, block, 0, st>>>(buf, bytes / 16, passes, ctx->d_scratch + 2);
    cudaEventRecord(b, st);
    ctx->launches.fetch_add(2);
    e = cudaGetLastError();
  }
  float ms = 0.0f;
  if (e == cudaSuccess) e = cudaEventSynchronize(b);
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  cudaFreeAsync(buf, st);
  if (e != cudaSuccess) return cuda_fail(e, "measure_l2_read");
  if (ms > 0.0f) *gb_s = (double)bytes * passes / (ms * 1e6);
  return MESO_OK;
}

meso_status meso_ctx_get_config(const meso_ctx* ctx, meso_config* out) {
  if (!ctx || !out) return fail(MESO_ERR_INVALID_ARG, "ctx_get_config: null argument");
  memset(out, 0, sizeof(*out));
  out->chunk_edge = 32;
  out->brick_edge = 8;
  out->device = ctx->device;
  out->mesh_ctas_per_sm = ctx->tuning.mesh_ctas_per_sm ? ctx->tuning.mesh_ctas_per_sm : 2;
  out->mesh_chunks_per_ticket = ctx->tuning.mesh_chunks_per_ticket ? ctx->tuning.mesh_chunks_per_ticket : 1;
  out->ray_tile_w = ctx->tuning.ray_tile_w ? ctx->tuning.ray_tile_w : 8;
  out->ray_tile_h = 32 / out->ray_tile_w;
  out->ray_warps_per_cta = ctx->tuning.ray_warps_per_cta ? ctx->tuning.ray_warps_per_cta : 4;
  out->hbm_budget_bytes = ctx->budget_bytes;
  out->tuning_path = nullptr;
  return MESO_OK;
}

uint64_t meso_kernel_launches(const meso_ctx* ctx) { return ctx ? ctx->launches.load() : 0; }
int meso_sm_count(const meso_ctx* ctx) { return ctx ? ctx->sm_count : 0; }

meso_status meso_dev_alloc(meso_ctx* ctx, size_t bytes, void** d_ptr) {
  if (!ctx || !d_ptr) return fail(MESO_ERR_INVALID_ARG, "dev_alloc: null argument");
  MESO_CUDA_TRY(cudaMalloc(d_ptr, bytes ? bytes : 16));
  return MESO_OK;
}
meso_status meso_dev_free(meso_ctx* ctx, void* d_ptr) {
  (void)ctx;
  MESO_CUDA_TRY(cudaFree(d_ptr));
  return MESO_OK;
}
meso_status meso_host_alloc_pinned(meso_ctx* ctx, size_t bytes, void** h_ptr) {
  if (!ctx || !h_ptr) return fail(MESO_ERR_INVALID_ARG, "host_alloc_pinned: null argument");
  MESO_CUDA_TRY(cudaMallocHost(h_ptr, bytes ? bytes : 16));
  return MESO_OK;
}
meso_status meso_host_free_pinned(meso_ctx* ctx, void* h_ptr) {
  (void)ctx;
  MESO_CUDA_TRY(cudaFreeHost(h_ptr));
  return MESO_OK;
}
meso_status meso_memcpy_h2d(meso_ctx* ctx, void* d_dst, const void* h_src, size_t bytes, void* stream) {
  MESO_CUDA_TRY(cudaMemcpyAsync(d_dst, h_src, bytes, cudaMemcpyHostToDevice, pick_stream(ctx, stream)));
  return MESO_OK;
}
meso_status meso_memcpy_d2h(meso_ctx* ctx, void* h_dst, const void* d_src, size_t bytes, void* stream) {
  MESO_CUDA_TRY(cudaMemcpyAsync(h_dst, d_src, bytes, cudaMemcpyDeviceToHost, pick_stream(ctx, stream)));
  return MESO_OK;
}
meso_status meso_memset(meso_ctx* ctx, void* d_dst, int value, size_t bytes, void* stream) {
  MESO_CUDA_TRY(cudaMemsetAsync(d_dst, value, bytes, pick_stream(ctx, stream)));
  return MESO_OK;
}
meso_status meso_stream_create(meso_ctx* ctx, void** stream) {
  (void)ctx;
  cudaStream_t s;
  MESO_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  *stream = s;
  return MESO_OK;
}
meso_status meso_stream_destroy(meso_ctx* ctx, void* stream) {
  (void)ctx;
  MESO_CUDA_TRY(cudaStreamDestroy((cudaStream_t)stream));
  return MESO_OK;
}
meso_status meso_event_create(meso_ctx* ctx, void** ev) {
  (void)ctx;
  cudaEvent_t e;
  MESO_CUDA_TRY(cudaEventCreate(&e));
  *ev = e;
  return MESO_OK;
}
meso_status meso_event_destroy(meso_ctx* ctx, void* ev) {
  (void)ctx;
  MESO_CUDA_TRY(cudaEventDestroy((cudaEvent_t)ev));
  return MESO_OK;
}
meso_status meso_event_record(meso_ctx* ctx, void* ev, void* stream) {
  MESO_CUDA_TRY(cudaEventRecord((cudaEvent_t)ev, pick_stream(ctx, stream)));
  return MESO_OK;
}
meso_status meso_event_elapsed_ms(meso_ctx* ctx, void* a, void* b, float* ms) {
  (void)ctx;
  MESO_CUDA_TRY(cudaEventSynchronize((cudaEvent_t)b));
  MESO_CUDA_TRY(cudaEventElapsedTime(ms, (cudaEvent_t)a, (cudaEvent_t)b));
  return MESO_OK;
}

// ---------------------------------------------------------------- scenes

meso_status meso_scene_create_terrain(meso_ctx* ctx, const meso_terrain* t, uint64_t spare, meso_scene** out) {
  if (!ctx) return fail(MESO_ERR_INVALID_ARG, "null ctx");
  std::lock_guard<std::mutex> lk(ctx->mu);
  return scene_create_terrain(ctx, t, spare, out);
}

meso_status meso_scene_create_dense(meso_ctx* ctx, const uint16_t* h_grid, int32_t nx, int32_t ny, int32_t nz,
                                    uint64_t spare, meso_scene** out) {
  if (!ctx) return fail(MESO_ERR_INVALID_ARG, "null ctx");
  std::lock_guard<std::mutex> lk(ctx->mu);
  return scene_create_dense(ctx, h_grid, nx, ny, nz, spare, out);
}

meso_status meso_scene_create_grid(meso_ctx* ctx, int32_t kind, const void* d_grid, int32_t nx, int32_t ny,
                                   int32_t nz, uint64_t spare, meso_scene** out) {
  if (!ctx) return fail(MESO_ERR_INVALID_ARG, "null ctx");
  std::lock_guard<std::mutex> lk(ctx->mu);
  return scene_create_grid(ctx, kind, d_grid, nx, ny, nz, spare, out);
}

meso_status meso_scene_count_solid(meso_ctx* ctx, const meso_scene* scene, uint64_t* n_solid) {
  if (!ctx) return fail(MESO_ERR_INVALID_ARG, "null ctx");
  return scene_count_solid(ctx, scene, n_solid);
}

meso_status meso_scene_destroy(meso_ctx* ctx, meso_scene* scene) {
  if (!ctx) return fail(MESO_ERR_INVALID_ARG, "null ctx");
  cudaDeviceSynchronize();
  scene_release(ctx, scene);
  return MESO_OK;
}

meso_status meso_scene_get_info(meso_ctx* ctx, const meso_scene* s, meso_scene_info* info) {
  if (!ctx || !s || !info) return fail(MESO_ERR_INVALID_ARG, "scene_get_info: null argument");
  int32_t alloc[2] = {0, 0};
  MESO_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  MESO_CUDA_TRY(cudaMemcpy(alloc, s->d_alloc, 8, cudaMemcpyDeviceToHost));
  info->nx = s->nx;
  info->ny = s->ny;
  info->nz = s->nz;
  info->n_bricks = (uint64_t)(alloc[0] - alloc[1]);
  info->brick_capacity = s->capacity;
  info->device_bytes = s->bytes;
  info->d_ptr = s->d_ptr;
  info->d_occ = s->d_occ;
  info->d_mat = s->d_mat;
  return MESO_OK;
}

meso_status meso_scene_download(meso_ctx* ctx, const meso_scene* s, uint32_t* h_ptr, uint64_t* h_occ,
                                uint16_t* h_mat) {
  if (!ctx || !s) return fail(MESO_ERR_INVALID_ARG, "scene_download: null argument");
  MESO_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  if (h_ptr) MESO_CUDA_TRY(cudaMemcpy(h_ptr, s->d_ptr, n_bricks_of(s) * 4, cudaMemcpyDeviceToHost));
  if (h_occ) MESO_CUDA_TRY(cudaMemcpy(h_occ, s->d_occ, s->capacity * 64, cudaMemcpyDeviceToHost));
  if (h_mat) MESO_CUDA_TRY(cudaMemcpy(h_mat, s->d_mat, s->capacity * 1024, cudaMemcpyDeviceToHost));
  return MESO_OK;
}

meso_status meso_generate_dense_u8(meso_ctx* ctx, int32_t nx, int32_t ny, int32_t nz, uint32_t seed, uint8_t* d_out,
                                   void* stream) {
  if (!ctx) return fail(MESO_ERR_INVALID_ARG, "null ctx");
  return generate_dense_u8(ctx, nx, ny, nz, seed, d_out, pick_stream(ctx, stream));
}

meso_status meso_generate_chunks_u16(meso_ctx* ctx, uint32_t n, uint32_t seed0, uint16_t* d_out, uint32_t* d_solid,
                                     void* stream) {
  if (!ctx) return fail(MESO_ERR_INVALID_ARG, "null ctx");
  return generate_chunks_u16(ctx, n, seed0, d_out, d_solid, pick_stream(ctx, stream));
}

// ---------------------------------------------------------------- meshing

meso_status meso_mesh_chunks(meso_ctx* ctx, const meso_mesh_source* src, const int32_t* d_coords, uint32_t n,
                             const meso_mesh_output* out, void* stream) {
  if (!ctx) return fail(MESO_ERR_INVALID_ARG, "null ctx");
  return launch_mesh(ctx, src, d_coords, n, out, pick_stream(ctx, stream), false);
}

meso_status meso_mesh_chunks_per_launch(meso_ctx* ctx, const meso_mesh_source* src, const int32_t* d_coords,
                                        uint32_t n, const meso_mesh_output* out, void* stream) {
  if (!ctx) return fail(MESO_ERR_INVALID_ARG, "null ctx");
  return launch_mesh(ctx, src, d_coords, n, out, pick_stream(ctx, stream), true);
}

meso_status meso_mesh_check(meso_ctx* ctx, const meso_mesh_output* out, void* stream, uint64_t* h_count) {
  if (!ctx || !out) return fail(MESO_ERR_INVALID_ARG, "mesh_check: null argument");
  cudaStream_t st = pick_stream(ctx, stream);
  uint64_t cnt = 0;
  MESO_CUDA_TRY(cudaMemcpyAsync(&cnt, out->d_quad_count, 8, cudaMemcpyDeviceToHost, st));
  MESO_CUDA_TRY(cudaStreamSynchronize(st));
  // the count is reported even when a device flag (e.g. a bad chunk
  // coordinate, whose chunk produced nothing) makes the call fail
  if (h_count) *h_count = cnt;
  MESO_TRY(meso_sync(ctx, st));
  if (cnt > out->capacity) return fail(MESO_ERR_OVERFLOW, "mesh: quad buffer too small");
  return MESO_OK;
}

}  // extern "C"

namespace {

// A contiguous host array of more than kHostSlice chunks is meshed in slices
// of kHostSlice chunks: the upload of slice i+1 (a second stream) overlaps
// the mesh launch of slice i, two device slice buffers in turn, and the
// launches append to one quad buffer with the chunks' indices in the whole
// array.  When h_quads is device-mapped page-locked memory the kernel writes
// the quads into it directly, over the CPU-GPU link while the next slice
// comes in the other way; otherwise they are copied back at the end.  On
// 4096 uint16 chunks with page-locked input and output: 2.11 ms in one
// upload, launch and download; slices of 256 / 512 / 1024 chunks 2.02 /
// 1.69 / 1.60 ms (a slice must fill the GPU's CTAs to mesh as fast as it
// arrives).
constexpr uint32_t kHostSlice = 1024;

meso_status mesh_host_pipelined(meso_ctx* ctx, int32_t kind, const uint8_t* h_data, uint32_t n, uint64_t* h_quads,
                                uint64_t capacity, uint64_t* h_count) {
  if (capacity && !h_quads) return fail(MESO_ERR_INVALID_ARG, "mesh_host: capacity without buffer");
  if (n > MESO_MAX_CHUNKS_PER_CALL) return fail(MESO_ERR_INVALID_ARG, "mesh_host: more than 2^20 chunks");
  const size_t chunk_bytes = kind == MESO_SRC_CHUNKS_U16 ? 65536 : 32768;
  const size_t slice_bytes = chunk_bytes * kHostSlice;
  const cudaStream_t st = ctx->stream;
  uint64_t* d_direct = nullptr;  // h_quads as the device sees it, if it can
  if (h_quads && capacity) {
    cudaPointerAttributes pa;
    if (cudaPointerGetAttributes(&pa, h_quads) == cudaSuccess && pa.type == cudaMemoryTypeHost && pa.devicePointer &&
        !(reinterpret_cast<uintptr_t>(pa.devicePointer) & 7u))
      d_direct = static_cast<uint64_t*>(pa.devicePointer);
    else
      cudaGetLastError();
  }
  cudaStream_t cs = nullptr;
  cudaEvent_t copied[2] = {nullptr, nullptr}, used[2] = {nullptr, nullptr}, ready = nullptr;
  uint8_t* d = nullptr;
  meso_status rc = MESO_OK;
  cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  for (int b = 0; b < 2 && e == cudaSuccess; b++) {
    e = cudaEventCreateWithFlags(&copied[b], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&used[b], cudaEventDisableTiming);
  }
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ready, cudaEventDisableTiming);
  // [0, 2 slices) inputs, then the count, then the quads unless written to host memory
  const size_t off_count = 2 * slice_bytes, off_quads = off_count + 256;
  const size_t total = off_quads + (d_direct ? 0 : capacity * 8);
  if (e == cudaSuccess) e = cudaMallocAsync(&d, total, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(d + off_count, 0, 8, st);
  if (e == cudaSuccess) e = cudaEventRecord(ready, st);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(cs, ready, 0);  // the buffers exist before the first copy
  if (e != cudaSuccess) rc = cuda_fail(e, "mesh_host: set-up");
  meso_mesh_output o;
  o.d_quads = d_direct ? d_direct : reinterpret_cast<uint64_t*>(d + off_quads);
  o.capacity = capacity;
  o.d_quad_count = reinterpret_cast<uint64_t*>(d + off_count);
  o.d_chunk_quad_counts = nullptr;
  for (uint32_t s0 = 0, i = 0; rc == MESO_OK && s0 < n; s0 += kHostSlice, i++) {
    const uint32_t cnt = n - s0 < kHostSlice ? n - s0 : kHostSlice;
    const int b = (int)(i & 1u);
    uint8_t* buf = d + (size_t)b * slice_bytes;
    if (i >= 2) e = cudaStreamWaitEvent(cs, used[b], 0);  // the launch of slice i-2 has read buf
    if (e == cudaSuccess) e = cudaMemcpyAsync(buf, h_data + (size_t)s0 * chunk_bytes, cnt * chunk_bytes,
                                              cudaMemcpyHostToDevice, cs);
    if (e == cudaSuccess) e = cudaEventRecord(copied[b], cs);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(st, copied[b], 0);
    if (e != cudaSuccess) {
      rc = cuda_fail(e, "mesh_host: upload");
      break;
    }
    meso_mesh_source src;
    memset(&src, 0, sizeof(src));
    src.kind = kind;
    src.d_data = buf;
    src.nx = (int32_t)cnt;
    rc = launch_mesh(ctx, &src, nullptr, cnt, &o, st, false, s0, true);
    if (rc == MESO_OK && (e = cudaEventRecord(used[b], st)) != cudaSuccess) rc = cuda_fail(e, "mesh_host: event");
  }
  uint64_t cnt = 0;
  if (rc == MESO_OK) {
    e = cudaMemcpyAsync(&cnt, o.d_quad_count, 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = cuda_fail(e, "mesh_host");
  }
  if (rc == MESO_OK && !d_direct && h_quads && capacity) {
    const uint64_t k = cnt < capacity ? cnt : capacity;
    e = cudaMemcpyAsync(h_quads, o.d_quads, k * 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = cuda_fail(e, "mesh_host download");
  }
  // everything issued on cs is ordered before work on st that has finished
  // or been synchronized; wait for cs too before its buffers and events go
  if (cs) cudaStreamSynchronize(cs);
  if (d) cudaFreeAsync(d, st);
  const meso_status sync_rc = meso_sync(ctx, st);
  if (rc == MESO_OK) rc = sync_rc;
  for (int b = 0; b < 2; b++) {
    if (copied[b]) cudaEventDestroy(copied[b]);
    if (used[b]) cudaEventDestroy(used[b]);
  }
  if (ready) cudaEventDestroy(ready);
  if (cs) cudaStreamDestroy(cs);
  if (h_count) *h_count = cnt;
  if (rc == MESO_OK && cnt > capacity) rc = fail(MESO_ERR_OVERFLOW, "mesh_host: quad buffer too small");
  return rc;
}

}  // namespace

extern "C" {

meso_status meso_mesh_host(meso_ctx* ctx, int32_t kind, const void* h_data, int32_t nx, int32_t ny, int32_t nz,
                           const int32_t* h_coords, uint32_t n, uint64_t* h_quads, uint64_t capacity,
                           uint64_t* h_count) {
  if (!ctx || !h_data) return fail(MESO_ERR_INVALID_ARG, "mesh_host: null argument");
  size_t data_bytes;
  size_t coord_bytes = 0;
  switch (kind) {
    case MESO_SRC_CHUNKS_U16:
      if (nx <= 0) nx = (int32_t)n;
      data_bytes = (size_t)nx * 65536;
      coord_bytes = h_coords ? 4ull * n : 0;
      break;
    case MESO_SRC_CHUNKS_U8:
      if (nx <= 0) nx = (int32_t)n;
      data_bytes = (size_t)nx * 32768;
      coord_bytes = h_coords ? 4ull * n : 0;
      break;
    case MESO_SRC_GRID_U8: data_bytes = (size_t)nx * ny * nz; coord_bytes = 12ull * n; break;
    case MESO_SRC_GRID_U16: data_bytes = (size_t)nx * ny * nz * 2; coord_bytes = 12ull * n; break;
    default: return fail(MESO_ERR_INVALID_ARG, "mesh_host: brick-map sources are device-resident; use meso_mesh_chunks");
  }
  if (coord_bytes && !h_coords) return fail(MESO_ERR_INVALID_ARG, "mesh_host: grid source needs coordinates");
  if ((kind == MESO_SRC_CHUNKS_U16 || kind == MESO_SRC_CHUNKS_U8) && !h_coords && n > kHostSlice)
    return mesh_host_pipelined(ctx, kind, static_cast<const uint8_t*>(h_data), n, h_quads, capacity, h_count);
  cudaStream_t st = ctx->stream;
  uint8_t* d = nullptr;
  const size_t off_coords = (data_bytes + 255) & ~size_t(255);
  const size_t off_count = (off_coords + coord_bytes + 255) & ~size_t(255);
  const size_t off_quads = off_count + 256;
  const size_t total = off_quads + capacity * 8;
  MESO_CUDA_TRY(cudaMallocAsync(&d, total, st));
  meso_status rc = MESO_OK;
  cudaError_t e = cudaMemcpyAsync(d, h_data, data_bytes, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && coord_bytes) e = cudaMemcpyAsync(d + off_coords, h_coords, coord_bytes, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) rc = cuda_fail(e, "mesh_host upload");
  meso_mesh_source src;
  memset(&src, 0, sizeof(src));
  src.kind = kind;
  src.d_data = d;
  src.nx = nx;
  src.ny = ny;
  src.nz = nz;
  meso_mesh_output o;
  o.d_quads = reinterpret_cast<uint64_t*>(d + off_quads);
  o.capacity = capacity;
  o.d_quad_count = reinterpret_cast<uint64_t*>(d + off_count);
  o.d_chunk_quad_counts = nullptr;
  if (rc == MESO_OK)
    rc = launch_mesh(ctx, &src, coord_bytes ? reinterpret_cast<const int32_t*>(d + off_coords) : nullptr, n, &o, st,
                     false);
  uint64_t cnt = 0;
  if (rc == MESO_OK) {
    e = cudaMemcpyAsync(&cnt, o.d_quad_count, 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = cuda_fail(e, "mesh_host");
  }
  if (rc == MESO_OK && h_quads && capacity) {
    const uint64_t k = cnt < capacity ? cnt : capacity;
    e = cudaMemcpyAsync(h_quads, o.d_quads, k * 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = cuda_fail(e, "mesh_host download");
  }
  cudaFreeAsync(d, st);
  if (rc == MESO_OK) rc = meso_sync(ctx, st);
  if (h_count) *h_count = cnt;
  if (rc == MESO_OK && cnt > capacity) rc = fail(MESO_ERR_OVERFLOW, "mesh_host: quad buffer too small");
  return rc;
}

// -------------------------------------------------------------- raymarching

meso_status meso_raymarch(meso_ctx* ctx, const meso_scene* const* scenes, const meso_camera* cams, uint32_t n_views,
                          const float light[3], uint32_t flags, meso_hit* d_hits, void* stream) {
  if (!ctx) return fail(MESO_ERR_INVALID_ARG, "null ctx");
  cudaStream_t st = pick_stream(ctx, stream);
  if (n_views <= 32) return launch_raymarch(ctx, scenes, cams, n_views, light, flags, d_hits, st, nullptr, 0);
  const size_t tb = raymarch_view_table_bytes(n_views);
  void* d_table = nullptr;
  MESO_CUDA_TRY(cudaMallocAsync(&d_table, tb, st));
  meso_status rc = launch_raymarch(ctx, scenes, cams, n_views, light, flags, d_hits, st, d_table, tb);
  cudaFreeAsync(d_table, st);
  return rc;
}

meso_status meso_raymarch_per_view(meso_ctx* ctx, const meso_scene* const* scenes, const meso_camera* cams,
                                   uint32_t n_views, const float light[3], uint32_t flags, meso_hit* d_hits,
                                   void* stream) {
  if (!ctx || !cams) return fail(MESO_ERR_INVALID_ARG, "raymarch_per_view: null argument");
  cudaStream_t st = pick_stream(ctx, stream);
  uint64_t off = 0;
  for (uint32_t v = 0; v < n_views; v++) {
    MESO_TRY(launch_raymarch(ctx, scenes + v, cams + v, 1, light, flags, d_hits + off, st, nullptr, 0));
    off += (uint64_t)cams[v].width * cams[v].height;
  }
  return MESO_OK;
}

meso_status meso_raymarch_host(meso_ctx* ctx, const meso_scene* scene, const meso_camera* cam, const float light[3],
                               uint32_t flags, meso_hit* h_hits) {
  if (!ctx || !scene || !cam || !h_hits) return fail(MESO_ERR_INVALID_ARG, "raymarch_host: null argument");
  cudaStream_t st = ctx->stream;
  const size_t n = (size_t)cam->width * cam->height;
  // Page-locked, device-mapped output: the kernel stores the hits straight
  // into host memory over the CPU-GPU link, overlapped with the tracing, so
  // there is no separate copy.  Pageable output: device buffer, one copy.
  cudaPointerAttributes pa;
  const bool mapped = cudaPointerGetAttributes(&pa, h_hits) == cudaSuccess && pa.type == cudaMemoryTypeHost &&
                      pa.devicePointer != nullptr;
  if (!mapped) cudaGetLastError();
  if (mapped) {
    meso_status rc = launch_raymarch(ctx, &scene, cam, 1, light, flags, static_cast<meso_hit*>(pa.devicePointer), st,
                                     nullptr, 0, nullptr, nullptr, nullptr, true);
    cudaError_t e = cudaStreamSynchronize(st);
    if (rc == MESO_OK && e != cudaSuccess) rc = cuda_fail(e, "raymarch_host");
    return rc;
  }
  meso_hit* d = nullptr;
  MESO_CUDA_TRY(cudaMallocAsync(&d, n * sizeof(meso_hit), st));
  meso_status rc = launch_raymarch(ctx, &scene, cam, 1, light, flags, d, st, nullptr, 0);
  if (rc == MESO_OK) {
    cudaError_t e = cudaMemcpyAsync(h_hits, d, n * sizeof(meso_hit), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = cuda_fail(e, "raymarch_host");
  }
  cudaFreeAsync(d, st);
  return rc;
}

meso_status meso_raymarch_stats(meso_ctx* ctx, const meso_scene* const* scenes, const meso_camera* cams,
                                uint32_t n_views, const float light[3], uint32_t flags, meso_hit* d_hits,
                                uint64_t h_counts[4]) {
  if (!ctx || !h_counts) return fail(MESO_ERR_INVALID_ARG, "raymarch_stats: null argument");
  if (n_views > 32) return fail(MESO_ERR_INVALID_ARG, "raymarch_stats: at most 32 views");
  cudaStream_t st = ctx->stream;
  uint64_t* d = nullptr;
  MESO_CUDA_TRY(cudaMallocAsync(&d, 32, st));
  MESO_CUDA_TRY(cudaMemsetAsync(d, 0, 32, st));
  meso_status rc = launch_raymarch(ctx, scenes, cams, n_views, light, flags, d_hits, st, nullptr, 0, d);
  if (rc == MESO_OK) {
    cudaError_t e = cudaMemcpyAsync(h_counts, d, 32, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = cuda_fail(e, "raymarch_stats");
  }
  cudaFreeAsync(d, st);
  return rc;
}

// ------------------------------------------------------------------- edits

meso_status meso_edit_spheres(meso_ctx* ctx, meso_scene* scene, const meso_sphere_edit* h_spheres, uint32_t n,
                              uint32_t* h_dirty, uint32_t dirty_cap, uint32_t* n_dirty, void* stream) {
  if (!ctx) return fail(MESO_ERR_INVALID_ARG, "null ctx");
  return edit_spheres(ctx, scene, h_spheres, n, h_dirty, dirty_cap, n_dirty, pick_stream(ctx, stream));
}

// ------------------------------------------------------------------ graphs

struct meso_graph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

meso_status meso_capture_begin(meso_ctx* ctx, void* stream) {
  if (!ctx || !stream) return fail(MESO_ERR_INVALID_ARG, "capture_begin: needs a context and an explicit stream");
  MESO_CUDA_TRY(cudaStreamBeginCapture((cudaStream_t)stream, cudaStreamCaptureModeThreadLocal));
  return MESO_OK;
}

meso_status meso_capture_end(meso_ctx* ctx, void* stream, meso_graph** out) {
  if (!ctx || !stream || !out) return fail(MESO_ERR_INVALID_ARG, "capture_end: null argument");
  cudaGraph_t g = nullptr;
  MESO_CUDA_TRY(cudaStreamEndCapture((cudaStream_t)stream, &g));
  cudaGraphExec_t x = nullptr;
  const cudaError_t e = cudaGraphInstantiate(&x, g, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g);
    return cuda_fail(e, "capture_end: cudaGraphInstantiate");
  }
  meso_graph* mg = new meso_graph();
  mg->graph = g;
  mg->exec = x;
  *out = mg;
  return MESO_OK;
}

meso_status meso_graph_launch(meso_graph* graph, void* stream) {
  if (!graph) return fail(MESO_ERR_INVALID_ARG, "graph_launch: null graph");
  MESO_CUDA_TRY(cudaGraphLaunch(graph->exec, (cudaStream_t)stream));
  return MESO_OK;
}

meso_status meso_graph_destroy(meso_graph* graph) {
  if (!graph) return MESO_OK;
  if (graph->exec) cudaGraphExecDestroy(graph->exec);
  if (graph->graph) cudaGraphDestroy(graph->graph);
  delete graph;
  return MESO_OK;
}

}  // extern "C"
