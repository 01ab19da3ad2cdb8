// store.cu -- the resident mesh of a brick-map scene: one quad arena in
// device memory and a per-chunk segment table (offset, count, capacity),
// replaced chunk by chunk when edits dirty them.
//
// Stands in for the reference's pooled chunk output: FChunkPool::PushToPool
// allocates a slot per chunk and swaps the lookup table when a chunk is
// regenerated (Runtimes/Voxel/Chunk/ChunkPool.h:446-622), PushToBlockPool
// writes the chunk's block instances into the pool (ChunkPool.h:381-445), and
// the pools are uploaded for the GPU to draw (ChunkPool.h:653-679).  Here the
// chunks' quads stay on the device:
//  - an update meshes the listed chunks in one batched launch into a
//    temporary buffer (quads of all chunks interleaved, each tagged with its
//    index in the call), then one kernel places every chunk -- in its old
//    segment when the new quads fit, else at the arena's bump pointer with
//    25 % slack -- and a scatter kernel copies each quad into its chunk's
//    segment (order inside a segment is unspecified);
//  - when the bump pointer would pass the end of the arena the placement of
//    that chunk fails and is flagged; the host then compacts: it packs every
//    live segment into a new arena (grown if needed) in chunk order and
//    remeshes the chunks whose placement failed.
#include <algorithm>
#include <cstring>
#include <vector>

#include "meso_internal.h"

namespace meso {
namespace {

constexpr uint64_t kInvalidOff = ~0ull;
constexpr uint64_t kChunkFieldMask = (1ull << 44) - 1;  // quad bits below the chunk field

// d_state words
enum : int { ST_TOP = 0, ST_LIVE = 1, ST_FLAGS = 2 };
enum : unsigned long long { FL_ARENA_FULL = 1, FL_TEMP_FULL = 2 };

// Segment capacity for `need` quads: 25 % slack, a multiple of 8.
__host__ __device__ inline uint32_t slack_cap(uint32_t need) {
  const uint64_t c = ((uint64_t)need + (need >> 2) + 7) & ~7ull;
  return c > 0xFFFFFFF8ull ? 0xFFFFFFF8u : (uint32_t)c;
}

// One thread per chunk of the call: chooses where chunk i's quads go.
__global__ void place_kernel(const int32_t* coords, uint32_t n, int CX, int CY, const uint32_t* need_counts,
                             const unsigned long long* temp_count, uint64_t temp_cap, uint64_t arena_cap,
                             uint64_t* off, uint32_t* cnt, uint32_t* cap, unsigned long long* state,
                             uint64_t* base, uint32_t* fill) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t c = (uint64_t)coords[3 * i] + (uint64_t)CX * ((uint64_t)coords[3 * i + 1] + (uint64_t)CY * coords[3 * i + 2]);
  fill[i] = 0;
  if (*temp_count > temp_cap) {  // the temporary buffer missed quads: place nothing
    base[i] = kInvalidOff;
    if (i == 0) atomicOr(state + ST_FLAGS, FL_TEMP_FULL);
    return;
  }
  const uint32_t need = need_counts[i];
  const uint32_t old = cnt[c];
  uint64_t o = off[c];
  if (o == kInvalidOff || need > cap[c]) {
    const uint32_t nc = slack_cap(need);
    const unsigned long long at = atomicAdd(state + ST_TOP, (unsigned long long)nc);
    if (at + nc <= arena_cap) {
      o = at;
      cap[c] = nc;
    } else {
      o = kInvalidOff;
      cap[c] = 0;
      atomicOr(state + ST_FLAGS, FL_ARENA_FULL);
    }
    off[c] = o;
  }
  cnt[c] = need;
  base[i] = o;
  atomicAdd(state + ST_LIVE, (unsigned long long)((long long)need - (long long)old));
}

// Copies each quad of the temporary buffer into its chunk's segment, with
// the chunk field cleared (the segment names the chunk).
// Every index is checked: a quad whose chunk field is not a chunk of the
// call, or one more quad than the chunk's count, is dropped, so no write can
// leave the chunk's segment.
__global__ void scatter_kernel(const uint64_t* temp, const unsigned long long* temp_count, uint64_t temp_cap,
                               uint32_t n, const uint32_t* need_counts, const uint64_t* base, uint32_t* fill,
                               uint64_t* arena, uint64_t arena_cap) {
  const uint64_t total = *temp_count;
  if (total > temp_cap) return;
  for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < total; k += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t q = temp[k];
    const uint32_t i = (uint32_t)(q >> 44);
    if (i >= n) continue;
    const uint64_t b = base[i];
    if (b == kInvalidOff) continue;
    const uint32_t pos = atomicAdd(fill + i, 1u);
    if (pos >= need_counts[i] || b + pos >= arena_cap) continue;
    arena[b + pos] = q & kChunkFieldMask;
  }
}

// Warp per chunk: moves live segments into a new arena at new offsets.
__global__ void compact_kernel(const uint64_t* old_arena, const uint64_t* old_off, const uint64_t* new_off,
                               const uint32_t* cnt, uint64_t n_chunks, uint64_t* new_arena) {
  const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
  const int lane = threadIdx.x & 31;
  for (uint64_t c = blockIdx.x * (uint64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); c < n_chunks; c += warps) {
    const uint64_t o = old_off[c];
    if (o == kInvalidOff) continue;
    const uint64_t d = new_off[c];
    const uint32_t k = cnt[c];
    for (uint32_t j = lane; j < k; j += 32) new_arena[d + j] = old_arena[o + j];
  }
}

// Gathers the segments of the listed chunks (k-th chunk's quads get chunk
// field k) into out at the given exclusive offsets; warp per chunk.
__global__ void gather_kernel(const uint64_t* arena, const uint64_t* off, const uint32_t* cnt, const uint32_t* list,
                              uint32_t n, const uint64_t* out_off, uint64_t cap, uint64_t* out) {
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  const int lane = threadIdx.x & 31;
  for (uint32_t k = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); k < n; k += warps) {
    const uint32_t c = list[k];
    const uint64_t o = off[c];
    if (o == kInvalidOff) continue;
    const uint32_t m = cnt[c];
    const uint64_t d = out_off[k];
    const uint64_t tag = (uint64_t)(k & 0xFFFFFu) << 44;
    for (uint32_t j = lane; j < m; j += 32)
      if (d + j < cap) out[d + j] = arena[o + j] | tag;
  }
}

}  // namespace
}  // namespace meso

struct meso_mesh_store {
  const meso_scene* scene = nullptr;
  int CX = 0, CY = 0, CZ = 0;
  uint64_t n_chunks = 0;
  uint64_t arena_cap = 0;
  uint64_t* d_arena = nullptr;
  uint64_t* d_off = nullptr;
  uint32_t* d_cnt = nullptr;
  uint32_t* d_cap = nullptr;
  unsigned long long* d_state = nullptr;  // top, live, flags
  uint64_t compactions = 0;
};

namespace meso {

meso_status store_place_async(meso_ctx* ctx, meso_mesh_store* S, const int32_t* d_coords, uint32_t n,
                              const uint64_t* d_temp, uint64_t temp_cap, const unsigned long long* d_temp_count,
                              const uint32_t* d_counts, void* d_work, cudaStream_t st) {
  if (n == 0) return MESO_OK;
  uint64_t* base = static_cast<uint64_t*>(d_work);
  uint32_t* fill = reinterpret_cast<uint32_t*>(base + n);
  place_kernel<<<(n + 255) / 256, 256, 0, st>>>(d_coords, n, S->CX, S->CY, d_counts, d_temp_count, temp_cap,
                                                S->arena_cap, S->d_off, S->d_cnt, S->d_cap, S->d_state, base, fill);
  scatter_kernel<<<ctx->sm_count * 8, 256, 0, st>>>(d_temp, d_temp_count, temp_cap, n, d_counts, base, fill,
                                                    S->d_arena, S->arena_cap);
  ctx->launches.fetch_add(2);
  MESO_CUDA_TRY(cudaGetLastError());
  return MESO_OK;
}

unsigned long long* store_flags_word(meso_mesh_store* S) { return S->d_state + ST_FLAGS; }

uint64_t store_device_bytes(const meso_mesh_store* S) {
  return S->arena_cap * 8 + S->n_chunks * 16 + 3 * sizeof(unsigned long long);
}

// Remeshes the n chunks at d_coords into the temporary buffer and places
// them (stream-ordered, no host wait).  d_work must hold n * 12 bytes.
static meso_status store_update_async(meso_ctx* ctx, meso_mesh_store* S, const int32_t* d_coords, uint32_t n,
                                      uint64_t* d_temp, uint64_t temp_cap, unsigned long long* d_temp_count,
                                      uint32_t* d_counts, void* d_work, cudaStream_t st) {
  if (n == 0) return MESO_OK;
  meso_mesh_source src;
  memset(&src, 0, sizeof(src));
  src.kind = MESO_SRC_BRICKMAP;
  src.scene = S->scene;
  meso_mesh_output o;
  o.d_quads = d_temp;
  o.capacity = temp_cap;
  o.d_quad_count = reinterpret_cast<uint64_t*>(d_temp_count);
  o.d_chunk_quad_counts = d_counts;
  MESO_TRY(launch_mesh(ctx, &src, d_coords, n, &o, st, false));
  return store_place_async(ctx, S, d_coords, n, d_temp, temp_cap, d_temp_count, d_counts, d_work, st);
}

// Reads and clears the store's flags (waits for st).
static meso_status read_flags(meso_mesh_store* S, cudaStream_t st, unsigned long long* flags) {
  MESO_CUDA_TRY(cudaMemcpyAsync(flags, S->d_state + ST_FLAGS, 8, cudaMemcpyDeviceToHost, st));
  MESO_CUDA_TRY(cudaMemsetAsync(S->d_state + ST_FLAGS, 0, 8, st));
  MESO_CUDA_TRY(cudaStreamSynchronize(st));
  return MESO_OK;
}

// Packs every live segment into a new arena in chunk order (capacity with
// slack, at least min_cap quads), frees the old one, and returns the chunks
// whose placement had failed (they hold a count but no segment).
static meso_status compact(meso_ctx* ctx, meso_mesh_store* S, uint64_t min_cap, cudaStream_t st,
                           std::vector<uint32_t>& unplaced) {
  const uint64_t N = S->n_chunks;
  std::vector<uint64_t> off(N), noff(N, kInvalidOff);
  std::vector<uint32_t> cnt(N), ncap(N, 0);
  MESO_CUDA_TRY(cudaStreamSynchronize(st));
  MESO_CUDA_TRY(cudaMemcpy(off.data(), S->d_off, N * 8, cudaMemcpyDeviceToHost));
  MESO_CUDA_TRY(cudaMemcpy(cnt.data(), S->d_cnt, N * 4, cudaMemcpyDeviceToHost));
  uint64_t top = 0;
  unplaced.clear();
  for (uint64_t c = 0; c < N; c++) {
    if (off[c] == kInvalidOff) {
      // a chunk whose placement failed gets its segment when it is placed again
      if (cnt[c]) unplaced.push_back((uint32_t)c);
      continue;
    }
    ncap[c] = slack_cap(cnt[c]);
    noff[c] = top;
    top += ncap[c];
  }
  const uint64_t cap = std::max<uint64_t>({min_cap, top + top / 2 + 4096, S->arena_cap});
  uint64_t* na = nullptr;
  uint64_t* d_noff = nullptr;
  MESO_CUDA_TRY(cudaMallocAsync(&na, cap * 8, st));
  cudaError_t e = cudaMallocAsync(&d_noff, N * 8, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_noff, noff.data(), N * 8, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    compact_kernel<<<ctx->sm_count * 8, 256, 0, st>>>(S->d_arena, S->d_off, d_noff, S->d_cnt, N, na);
    ctx->launches.fetch_add(1);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(S->d_off, noff.data(), N * 8, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(S->d_cap, ncap.data(), N * 4, cudaMemcpyHostToDevice, st);
  unsigned long long state[3] = {top, 0, 0};
  uint64_t live = 0;
  for (uint64_t c = 0; c < N; c++)
    if (noff[c] != kInvalidOff) live += cnt[c];
  state[ST_LIVE] = live;
  // unplaced chunks' counts are re-added when they are placed
  for (uint32_t c : unplaced) cnt[c] = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(S->d_cnt, cnt.data(), N * 4, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(S->d_state, state, sizeof(state), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    cudaFreeAsync(na, st);
    cudaFreeAsync(d_noff, st);
    cudaStreamSynchronize(st);
    return cuda_fail(e, "mesh store compaction");
  }
  cudaFreeAsync(S->d_arena, st);
  cudaFreeAsync(d_noff, st);
  S->d_arena = na;
  S->arena_cap = cap;
  S->compactions++;
  MESO_CUDA_TRY(cudaStreamSynchronize(st));
  return MESO_OK;
}

// Remeshes the chunks (linear indices) and waits until the store holds
// them, compacting and retrying as often as the arena or the temporary
// buffer requires.
meso_status store_update_sync(meso_ctx* ctx, meso_mesh_store* S, const uint32_t* h_chunks, uint32_t n,
                              cudaStream_t st) {
  // a chunk listed twice would be placed twice at once: keep one of each
  std::vector<uint32_t> todo(h_chunks, h_chunks + n);
  std::sort(todo.begin(), todo.end());
  todo.erase(std::unique(todo.begin(), todo.end()), todo.end());
  uint64_t temp_cap = 0;
  for (int round = 0; round < 8 && !todo.empty(); round++) {
    for (uint32_t c : todo)
      if (c >= S->n_chunks) return fail(MESO_ERR_INVALID_ARG, "mesh store: chunk index outside the scene");
    // in batches of at most 2^20 chunks (the quad's chunk field)
    std::vector<uint32_t> failed;
    for (size_t b0 = 0; b0 < todo.size(); b0 += MESO_MAX_CHUNKS_PER_CALL) {
      const uint32_t m = (uint32_t)std::min<size_t>(todo.size() - b0, MESO_MAX_CHUNKS_PER_CALL);
      std::vector<int32_t> coords(3 * (size_t)m);
      for (uint32_t k = 0; k < m; k++) {
        const uint32_t c = todo[b0 + k];
        coords[3 * k] = (int32_t)(c % S->CX);
        coords[3 * k + 1] = (int32_t)((c / S->CX) % S->CY);
        coords[3 * k + 2] = (int32_t)(c / ((uint32_t)S->CX * S->CY));
      }
      if (temp_cap == 0) temp_cap = std::max<uint64_t>(4096, (uint64_t)m * 2048);
      uint8_t* d = nullptr;
      const size_t off_counts = ((size_t)12 * m + 255) & ~size_t(255);
      const size_t off_work = off_counts + (((size_t)4 * m + 255) & ~size_t(255));
      const size_t off_tc = off_work + (((size_t)16 * m + 8 + 255) & ~size_t(255));
      const size_t off_temp = off_tc + 256;
      MESO_CUDA_TRY(cudaMallocAsync(&d, off_temp + temp_cap * 8, st));
      cudaError_t e = cudaMemcpyAsync(d, coords.data(), 12ull * m, cudaMemcpyHostToDevice, st);
      meso_status rc = e == cudaSuccess ? MESO_OK : cuda_fail(e, "mesh store upload");
      if (rc == MESO_OK)
        rc = store_update_async(ctx, S, reinterpret_cast<const int32_t*>(d), m,
                                reinterpret_cast<uint64_t*>(d + off_temp), temp_cap,
                                reinterpret_cast<unsigned long long*>(d + off_tc),
                                reinterpret_cast<uint32_t*>(d + off_counts), d + off_work, st);
      unsigned long long tc = 0, flags = 0;
      if (rc == MESO_OK) {
        e = cudaMemcpyAsync(&tc, d + off_tc, 8, cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) rc = cuda_fail(e, "mesh store");
      }
      if (rc == MESO_OK) rc = read_flags(S, st, &flags);
      cudaFreeAsync(d, st);
      if (rc == MESO_OK) rc = meso_sync(ctx, st);
      if (rc != MESO_OK) return rc;
      if (flags & FL_TEMP_FULL) {
        // nothing of this batch was placed: retry it with a buffer that fits
        temp_cap = tc + tc / 8 + 4096;
        failed.insert(failed.end(), todo.begin() + b0, todo.begin() + b0 + m);
        continue;
      }
      if (flags & FL_ARENA_FULL) {
        std::vector<uint32_t> unplaced;
        MESO_TRY(compact(ctx, S, 0, st, unplaced));
        failed.insert(failed.end(), unplaced.begin(), unplaced.end());
      }
    }
    std::sort(failed.begin(), failed.end());
    failed.erase(std::unique(failed.begin(), failed.end()), failed.end());
    todo.swap(failed);
  }
  if (!todo.empty()) return fail(MESO_ERR_OOM, "mesh store: placement did not converge");
  return MESO_OK;
}

}  // namespace meso

using namespace meso;

extern "C" {

meso_status meso_mesh_store_create(meso_ctx* ctx, const meso_scene* scene, meso_mesh_store** out) {
  if (!ctx || !scene || !out) return fail(MESO_ERR_INVALID_ARG, "mesh_store_create: null argument");
  *out = nullptr;
  if (scene->nx % 32 || scene->ny % 32 || scene->nz % 32)
    return fail(MESO_ERR_INVALID_ARG, "mesh_store_create: scene dims must be multiples of 32");
  cudaStream_t st = ctx->stream;
  meso_mesh_store* S = new meso_mesh_store();
  S->scene = scene;
  S->CX = scene->nx / 32;
  S->CY = scene->ny / 32;
  S->CZ = scene->nz / 32;
  S->n_chunks = (uint64_t)S->CX * S->CY * S->CZ;
  const uint64_t N = S->n_chunks;
  // non-empty chunks: the scene's 4x4x4-brick cell map, one byte per chunk
  std::vector<uint8_t> macro(N);
  cudaError_t e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = cudaMemcpy(macro.data(), scene->d_macro, N, cudaMemcpyDeviceToHost);
  std::vector<uint32_t> chunks;
  for (uint64_t c = 0; c < N; c++)
    if (macro[c]) chunks.push_back((uint32_t)c);
  S->arena_cap = std::max<uint64_t>(65536, (uint64_t)chunks.size() * 1024);
  if (e == cudaSuccess) e = cudaMalloc(&S->d_arena, S->arena_cap * 8);
  if (e == cudaSuccess) e = cudaMalloc(&S->d_off, N * 8);
  if (e == cudaSuccess) e = cudaMalloc(&S->d_cnt, N * 4);
  if (e == cudaSuccess) e = cudaMalloc(&S->d_cap, N * 4);
  if (e == cudaSuccess) e = cudaMalloc(&S->d_state, 3 * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemsetAsync(S->d_off, 0xFF, N * 8, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(S->d_cnt, 0, N * 4, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(S->d_cap, 0, N * 4, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(S->d_state, 0, 3 * sizeof(unsigned long long), st);
  meso_status rc = e == cudaSuccess ? MESO_OK : cuda_fail(e, "mesh_store_create");
  if (rc == MESO_OK && !chunks.empty()) rc = store_update_sync(ctx, S, chunks.data(), (uint32_t)chunks.size(), st);
  if (rc != MESO_OK) {
    meso_mesh_store_destroy(ctx, S);
    return rc;
  }
  *out = S;
  return MESO_OK;
}

meso_status meso_mesh_store_update(meso_ctx* ctx, meso_mesh_store* store, const uint32_t* h_chunks, uint32_t n) {
  if (!ctx || !store || (n && !h_chunks)) return fail(MESO_ERR_INVALID_ARG, "mesh_store_update: null argument");
  return store_update_sync(ctx, store, h_chunks, n, ctx->stream);
}

meso_status meso_mesh_store_get_info(meso_ctx* ctx, const meso_mesh_store* store, meso_mesh_store_info* info) {
  if (!ctx || !store || !info) return fail(MESO_ERR_INVALID_ARG, "mesh_store_get_info: null argument");
  unsigned long long state[3] = {0, 0, 0};
  MESO_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  MESO_CUDA_TRY(cudaMemcpy(state, store->d_state, sizeof(state), cudaMemcpyDeviceToHost));
  memset(info, 0, sizeof(*info));
  info->n_chunks = store->n_chunks;
  info->live_quads = state[ST_LIVE];
  info->arena_quads = store->arena_cap;
  info->arena_used = state[ST_TOP];
  info->compactions = store->compactions;
  info->d_arena = store->d_arena;
  info->d_seg_offset = store->d_off;
  info->d_seg_count = store->d_cnt;
  return MESO_OK;
}

meso_status meso_mesh_store_gather(meso_ctx* ctx, const meso_mesh_store* store, const uint32_t* h_chunks, uint32_t n,
                                   uint64_t* d_out, uint64_t capacity, uint64_t* h_total) {
  if (!ctx || !store || (n && !h_chunks) || !h_total)
    return fail(MESO_ERR_INVALID_ARG, "mesh_store_gather: null argument");
  if (n > MESO_MAX_CHUNKS_PER_CALL) return fail(MESO_ERR_INVALID_ARG, "mesh_store_gather: more than 2^20 chunks");
  if (capacity && !d_out) return fail(MESO_ERR_INVALID_ARG, "mesh_store_gather: capacity without buffer");
  *h_total = 0;
  if (n == 0) return MESO_OK;
  for (uint32_t k = 0; k < n; k++)
    if (h_chunks[k] >= store->n_chunks) return fail(MESO_ERR_INVALID_ARG, "mesh_store_gather: chunk outside the scene");
  cudaStream_t st = ctx->stream;
  std::vector<uint32_t> cnt(store->n_chunks);
  MESO_CUDA_TRY(cudaStreamSynchronize(st));
  MESO_CUDA_TRY(cudaMemcpy(cnt.data(), store->d_cnt, store->n_chunks * 4, cudaMemcpyDeviceToHost));
  std::vector<uint64_t> offs(n);
  uint64_t total = 0;
  for (uint32_t k = 0; k < n; k++) {
    offs[k] = total;
    total += cnt[h_chunks[k]];
  }
  *h_total = total;
  uint8_t* d = nullptr;
  const size_t off_offs = ((size_t)4 * n + 255) & ~size_t(255);
  MESO_CUDA_TRY(cudaMallocAsync(&d, off_offs + 8ull * n, st));
  cudaError_t e = cudaMemcpyAsync(d, h_chunks, 4ull * n, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d + off_offs, offs.data(), 8ull * n, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && capacity) {
    gather_kernel<<<ctx->sm_count * 8, 256, 0, st>>>(store->d_arena, store->d_off, store->d_cnt,
                                                     reinterpret_cast<const uint32_t*>(d), n,
                                                     reinterpret_cast<const uint64_t*>(d + off_offs), capacity, d_out);
    ctx->launches.fetch_add(1);
    e = cudaGetLastError();
  }
  cudaFreeAsync(d, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "mesh_store_gather");
  if (total > capacity) return fail(MESO_ERR_OVERFLOW, "mesh_store_gather: output buffer too small");
  return MESO_OK;
}

meso_status meso_mesh_store_destroy(meso_ctx* ctx, meso_mesh_store* store) {
  if (!store) return MESO_OK;
  if (ctx) cudaStreamSynchronize(ctx->stream);
  cudaFree(store->d_arena);
  cudaFree(store->d_off);
  cudaFree(store->d_cnt);
  cudaFree(store->d_cap);
  cudaFree(store->d_state);
  delete store;
  return MESO_OK;
}

}  // extern "C"
