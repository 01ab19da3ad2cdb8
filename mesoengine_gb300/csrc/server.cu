// server.cu -- the serving loop: resident scenes, a request queue, and a
// native scheduler thread that batches requests onto a pool of CUDA streams
// as they arrive (continuous batching).
//
// Replaces the reference's host ThreadPool + double-buffered modify queue
// (Runtimes/Thread/ThreadPool.h:7-127, Runtimes/Thread/DoubleBufferQueue.h:4-51)
// and the per-frame dispatch of FChunkManage::UpdateLoadingQueue
// (Runtimes/Voxel/Chunk/ChunkManager.h:211-400), which throttles chunk work
// at MaxUnsyncedLoadChunkCount and re-queues a task when the pool is busy.
//
// Model:
//  - every in-flight batch owns a slot: a stream, a completion event and
//    device buffers sized at creation, all charged to the HBM budget; a batch
//    starts as soon as a slot is free (requests that arrive while others are
//    on the GPU join the next batch);
//  - render requests with the same flags are batched into ONE multi-view
//    raymarch launch (views may come from different scenes);
//  - an edit+remesh+render request runs alone in its slot; per scene,
//    requests start in arrival order around edits (a render that arrived
//    before an edit may run with other renders; one that arrived after waits
//    for the edit), so every result equals a sequential replay;
//  - results are summarised on the device (order-sensitive hash of the hit
//    buffer and traced shadow rays, computed by the raymarch kernel itself;
//    order-insensitive hash of the quads) and the hits can be kept for
//    meso_server_fetch_hits;
//  - a request's hits go straight to its dst_hits when that is device memory
//    of the server's device or device-mapped page-locked host memory (the
//    kernel's stores cross the CPU-GPU link while it traces); other
//    destinations get a copy from the batch buffer;
//  - a request that can never fit a slot, or that arrives when max_queue
//    requests are already waiting, completes at once with
//    MESO_ERR_OVER_BUDGET.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <thread>

#include <sys/prctl.h>
#include <unordered_map>
#include <vector>

#include "meso_internal.h"

namespace meso {
meso_status edit_spheres(meso_ctx*, meso_scene*, const meso_sphere_edit*, uint32_t, uint32_t*, uint32_t, uint32_t*,
                         cudaStream_t);
}

namespace meso {
namespace {

constexpr uint32_t kMaxBatch = 64;
static_assert(kMaxBatch == kRayHashViews, "the raymarch kernel sums checksums of at most one batch of views");
constexpr uint32_t kQuadHash = kRayHashEntries, kQuadCount = kRayHashEntries + 1, kSums = kRayHashEntries + 2;

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  // splitmix64 finaliser
  x ^= x >> 30;
  x *= 0xBF58476D1CE4E5B9ull;
  x ^= x >> 27;
  x *= 0x94D049BB133111EBull;
  x ^= x >> 31;
  return x;
}

// out[0] += sum mix64(q) over the min(count, cap) quads.
__global__ void quad_hash_kernel(const uint64_t* quads, const uint64_t* count, uint64_t cap,
                                 unsigned long long* out) {
  const uint64_t n = *count < cap ? *count : cap;
  unsigned long long acc = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    acc += mix64(quads[i]);
  for (int o = 16; o; o >>= 1) acc += __shfl_down_sync(0xFFFFFFFFu, acc, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, acc);
}

struct SrvRequest {
  uint64_t id = 0;
  meso_request req;
  std::vector<meso_sphere_edit> edits;
  double submit = 0;
  uint64_t pixels = 0;
  meso_hit* d_dst = nullptr;  // device address the kernel may store dst_hits through (null: copy)
  bool dst_host = false;      // d_dst is page-locked host memory
};

struct Slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  // edit batches: the render runs on stream2, forked after the edit and
  // joined before the results are read, so it overlaps the remesh
  cudaStream_t stream2 = nullptr;
  cudaEvent_t forked = nullptr, joined = nullptr;
  meso_hit* d_hits = nullptr;
  uint64_t hit_cap = 0;  // pixels
  void* d_table = nullptr;
  size_t table_bytes = 0;
  // [0, kRayHashEntries): the raymarch's partial hit hashes and shadow
  // counts; then the quad hash and the quad count
  unsigned long long* d_sums = nullptr;
  unsigned long long* h_sums = nullptr;  // pinned copy
  uint64_t* d_quads = nullptr;
  uint64_t quad_cap = 0;
  int32_t* d_coords = nullptr;
  int32_t* h_coords = nullptr;  // pinned staging
  uint32_t coord_cap = 0;
  // keep_meshes: per-chunk quad counts of the remesh, placement scratch
  // (12 bytes per chunk) and the store's flags copied back with the results
  uint32_t* d_counts = nullptr;
  void* d_place = nullptr;
  unsigned long long* h_flags = nullptr;
  meso_hit* h_hits = nullptr;  // pinned, keep_hits only
  bool busy = false;
  bool edit = false;
  std::vector<SrvRequest> reqs;
  std::vector<uint64_t> offsets;
  uint32_t n_dirty = 0;
  double start = 0;
  meso_status launch_status = MESO_OK;
};

uint64_t pixels_of(const meso_camera& c) { return (uint64_t)c.width * c.height; }

}  // namespace
}  // namespace meso

struct meso_server {
  meso_ctx* ctx = nullptr;
  meso_server_config cfg;
  float light[3];
  std::vector<meso_scene*> scenes;
  std::vector<meso::Slot> slots;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<meso::SrvRequest> queue;
  std::vector<meso_completion> done;
  std::unordered_map<uint64_t, std::vector<meso_hit>> kept;
  std::vector<int> scene_busy;        // in-flight batches touching the scene
  std::vector<int> scene_edit_busy;   // an edit of the scene is in flight
  std::atomic<bool> stop{false};
  std::thread th;
  uint64_t next_id = 1;
  uint64_t inflight = 0;
  std::chrono::steady_clock::time_point t0;
  std::vector<uint32_t> dirty;  // scratch for edit dirty lists
  std::vector<meso_mesh_store*> stores;  // keep_meshes: one per scene
  double now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
};

namespace meso {
namespace {

void release_slot(Slot& s) {
  if (s.stream) cudaStreamSynchronize(s.stream);
  cudaFree(s.d_hits);
  cudaFree(s.d_table);
  cudaFree(s.d_sums);
  cudaFree(s.d_quads);
  cudaFree(s.d_coords);
  cudaFree(s.d_counts);
  cudaFree(s.d_place);
  cudaFreeHost(s.h_flags);
  cudaFreeHost(s.h_sums);
  cudaFreeHost(s.h_coords);
  cudaFreeHost(s.h_hits);
  if (s.done) cudaEventDestroy(s.done);
  if (s.forked) cudaEventDestroy(s.forked);
  if (s.joined) cudaEventDestroy(s.joined);
  if (s.stream2) cudaStreamDestroy(s.stream2);
  if (s.stream) cudaStreamDestroy(s.stream);
  s = Slot();
}

meso_completion make_completion(meso_server* srv, const SrvRequest& r, meso_status st, double start) {
  meso_completion c;
  memset(&c, 0, sizeof(c));
  c.request_id = r.id;
  c.user_tag = r.req.user_tag;
  c.status = st;
  c.submit_s = r.submit;
  c.start_s = start;
  c.done_s = srv->now();
  return c;
}

// Forms the next batch from the queue (caller holds srv->mu).  Per scene,
// requests start in arrival order around edits.
bool form_batch(meso_server* srv, std::vector<SrvRequest>& out, bool& is_edit) {
  out.clear();
  is_edit = false;
  const uint32_t max_req = std::min<uint32_t>(srv->cfg.max_batch_requests ? srv->cfg.max_batch_requests : kMaxBatch,
                                              kMaxBatch);
  const uint64_t max_rays = srv->slots.empty() ? 0 : srv->slots[0].hit_cap;
  std::vector<char> blocked(srv->scenes.size(), 0);
  for (size_t s = 0; s < srv->scenes.size(); s++) blocked[s] = srv->scene_edit_busy[s] ? 1 : 0;
  uint64_t rays = 0;
  uint32_t flags = 0;
  for (auto it = srv->queue.begin(); it != srv->queue.end();) {
    const uint32_t sc = it->req.scene_index;
    const bool edit = it->req.kind == MESO_REQ_EDIT_REMESH_RENDER;
    if (blocked[sc]) {
      ++it;
      continue;
    }
    if (edit) {
      // an edit waits for every earlier request of its scene to finish
      if (out.empty() && srv->scene_busy[sc] == 0) {
        out.push_back(std::move(*it));
        srv->queue.erase(it);
        is_edit = true;
        return true;
      }
      blocked[sc] = 1;  // later requests of this scene wait for the edit
      ++it;
      continue;
    }
    if (!out.empty() && (it->req.flags != flags || out.size() >= max_req || rays + it->pixels > max_rays)) {
      ++it;
      continue;
    }
    if (out.empty()) flags = it->req.flags;
    rays += it->pixels;
    out.push_back(std::move(*it));
    it = srv->queue.erase(it);
    if (out.size() >= max_req) break;
  }
  return !out.empty();
}

void launch_batch(meso_server* srv, Slot& s) {
  meso_ctx* ctx = srv->ctx;
  const cudaStream_t st = s.stream;
  s.launch_status = MESO_OK;
  s.offsets.clear();
  s.n_dirty = 0;
  cudaMemsetAsync(s.d_sums, 0, sizeof(unsigned long long) * kSums, st);
  std::vector<const meso_scene*> scenes;
  std::vector<meso_camera> cams;
  std::vector<meso_hit*> view_out;
  bool direct = false, host_out = false;
  uint64_t off = 0;
  for (auto& r : s.reqs) {
    scenes.push_back(srv->scenes[r.req.scene_index]);
    cams.push_back(r.req.camera);
    view_out.push_back(r.d_dst);
    direct = direct || r.d_dst;
    host_out = host_out || r.dst_host;
    s.offsets.push_back(off);
    off += r.pixels;
  }
  meso_status rc = MESO_OK;
  const cudaStream_t rs = s.edit ? s.stream2 : st;  // the render's stream
  bool rendered = false;  // work was issued on rs: st must join it before the batch completes
  // the batch's render (one launch for all its views), then the copies into
  // the callers' buffers that the kernel could not store into, before the
  // completion is signalled
  auto render = [&]() {
    rendered = true;
    rc = launch_raymarch(ctx, scenes.data(), cams.data(), (uint32_t)cams.size(), srv->light, s.reqs[0].req.flags,
                         s.d_hits, rs, s.d_table, s.table_bytes, nullptr, direct ? view_out.data() : nullptr,
                         s.d_sums, host_out);
    if (rc != MESO_OK) return;
    for (size_t k = 0; k < s.reqs.size(); k++) {
      meso_hit* dst = s.reqs[k].req.dst_hits;
      if (dst && !s.reqs[k].d_dst)
        cudaMemcpyAsync(dst, s.d_hits + s.offsets[k], s.reqs[k].pixels * sizeof(meso_hit), cudaMemcpyDefault, rs);
    }
  };
  if (s.edit) {
    SrvRequest& r = s.reqs[0];
    meso_scene* scene = srv->scenes[r.req.scene_index];
    uint32_t n_dirty = 0;
    rc = edit_spheres(ctx, scene, r.edits.data(), (uint32_t)r.edits.size(), srv->dirty.data(),
                      (uint32_t)srv->dirty.size(), &n_dirty, st);
    if (rc == MESO_OK) {
      // the render needs only the edited scene: it is issued first, on the
      // second stream, and the remesh runs beside it
      cudaEventRecord(s.forked, st);
      cudaStreamWaitEvent(s.stream2, s.forked, 0);
      render();
    }
    if (rc == MESO_OK && n_dirty > s.coord_cap) rc = fail(MESO_ERR_OVERFLOW, "server: too many dirty chunks");
    if (rc == MESO_OK && n_dirty) {
      const int CX = scene->nx / 32, CY = scene->ny / 32;
      for (uint32_t k = 0; k < n_dirty; k++) {
        const uint32_t c = srv->dirty[k];
        s.h_coords[3 * k] = (int32_t)(c % CX);
        s.h_coords[3 * k + 1] = (int32_t)((c / CX) % CY);
        s.h_coords[3 * k + 2] = (int32_t)(c / ((uint32_t)CX * CY));
      }
      cudaMemcpyAsync(s.d_coords, s.h_coords, 12ull * n_dirty, cudaMemcpyHostToDevice, st);
      meso_mesh_source src;
      memset(&src, 0, sizeof(src));
      src.kind = MESO_SRC_BRICKMAP;
      src.scene = scene;
      meso_mesh_output o;
      o.d_quads = s.d_quads;
      o.capacity = s.quad_cap;
      o.d_quad_count = reinterpret_cast<uint64_t*>(s.d_sums + kQuadCount);
      meso_mesh_store* store = srv->stores.empty() ? nullptr : srv->stores[r.req.scene_index];
      o.d_chunk_quad_counts = store ? s.d_counts : nullptr;
      rc = launch_mesh(ctx, &src, s.d_coords, n_dirty, &o, st, false);
      if (rc == MESO_OK) {
        quad_hash_kernel<<<64, 256, 0, st>>>(s.d_quads, o.d_quad_count, s.quad_cap, s.d_sums + kQuadHash);
        ctx->launches.fetch_add(1);
      }
      // the scene's resident mesh: the dirty chunks' new quads replace their
      // segments; a failed placement is flagged and repaired at completion
      if (rc == MESO_OK && store)
        rc = store_place_async(ctx, store, s.d_coords, n_dirty, s.d_quads, s.quad_cap,
                               reinterpret_cast<const unsigned long long*>(o.d_quad_count), s.d_counts, s.d_place,
                               st);
      if (rc == MESO_OK && store) {
        cudaMemcpyAsync(s.h_flags, store_flags_word(store), sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
        cudaMemsetAsync(store_flags_word(store), 0, sizeof(unsigned long long), st);
      }
    }
    s.n_dirty = n_dirty;
  } else {
    render();
  }
  if (s.edit && rendered) {
    // whatever was issued on the render's stream completes before the batch
    cudaEventRecord(s.joined, rs);
    cudaStreamWaitEvent(st, s.joined, 0);
  }
  if (rc == MESO_OK) {
    cudaMemcpyAsync(s.h_sums, s.d_sums, sizeof(unsigned long long) * kSums, cudaMemcpyDeviceToHost, st);
    if (srv->cfg.keep_hits) cudaMemcpyAsync(s.h_hits, s.d_hits, off * sizeof(meso_hit), cudaMemcpyDeviceToHost, st);
  }
  if (rc == MESO_OK) {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) rc = cuda_fail(e, "server: batch launch");
  }
  s.launch_status = rc;
  cudaEventRecord(s.done, st);
}

// A remesh whose placement in the scene's mesh store failed (full arena or
// temporary buffer) is placed again, synchronously, before the scene's next
// request may start.
meso_status repair_store(meso_server* srv, Slot& s) {
  meso_mesh_store* store = srv->stores[s.reqs[0].req.scene_index];
  const meso_scene* scene = srv->scenes[s.reqs[0].req.scene_index];
  const uint32_t CX = (uint32_t)scene->nx / 32, CY = (uint32_t)scene->ny / 32;
  std::vector<uint32_t> chunks(s.n_dirty);
  for (uint32_t k = 0; k < s.n_dirty; k++)
    chunks[k] = (uint32_t)s.h_coords[3 * k] + CX * ((uint32_t)s.h_coords[3 * k + 1] + CY * (uint32_t)s.h_coords[3 * k + 2]);
  return store_update_sync(srv->ctx, store, chunks.data(), s.n_dirty, s.stream);
}

void finish_batch(meso_server* srv, Slot& s) {
  if (s.edit && s.launch_status == MESO_OK && !srv->stores.empty() && s.n_dirty && *s.h_flags) {
    *s.h_flags = 0;
    s.launch_status = repair_store(srv, s);
  }
  std::vector<meso_completion> comps;
  for (size_t k = 0; k < s.reqs.size(); k++) {
    const SrvRequest& r = s.reqs[k];
    meso_completion c = make_completion(srv, r, s.launch_status, s.start);
    if (s.launch_status == MESO_OK) {
      unsigned long long hh = 0, sh = 0;
      for (uint32_t j = 0; j < kRayHashSlots; j++) {
        hh += s.h_sums[k * kRayHashSlots + j];
        sh += s.h_sums[kRayHashShadow + k * kRayHashSlots + j];
      }
      c.hit_checksum = hh;
      c.n_rays = r.pixels + sh;
      if (s.edit) {
        c.n_dirty_chunks = s.n_dirty;
        c.quad_checksum = s.h_sums[kQuadHash];
        c.n_quads = s.n_dirty ? s.h_sums[kQuadCount] : 0;
        if (c.n_quads > s.quad_cap) c.status = MESO_ERR_OVERFLOW;
      }
    }
    comps.push_back(c);
  }
  std::lock_guard<std::mutex> lk(srv->mu);
  for (size_t k = 0; k < s.reqs.size(); k++) {
    const SrvRequest& r = s.reqs[k];
    srv->scene_busy[r.req.scene_index]--;
    if (s.edit) srv->scene_edit_busy[r.req.scene_index] = 0;
    if (srv->cfg.keep_hits && s.launch_status == MESO_OK)
      srv->kept[r.id] = std::vector<meso_hit>(s.h_hits + s.offsets[k], s.h_hits + s.offsets[k] + r.pixels);
    srv->done.push_back(comps[k]);
  }
  srv->inflight--;
  s.busy = false;
  s.reqs.clear();
  srv->cv.notify_all();
}

void scheduler(meso_server* srv) {
  cudaSetDevice(srv->ctx->device);
  // polling sleeps of a few microseconds need a fine timer slack for this
  // thread (the default of 50 us would stretch each one to ~70 us)
  prctl(PR_SET_TIMERSLACK, 1000UL, 0UL, 0UL, 0UL);
  std::vector<SrvRequest> batch;
  for (;;) {
    bool any_busy = false;
    for (auto& s : srv->slots) {
      if (!s.busy) continue;
      if (cudaEventQuery(s.done) == cudaSuccess) finish_batch(srv, s);
      else any_busy = true;
    }
    for (auto& s : srv->slots) {
      if (s.busy) continue;
      bool is_edit = false;
      {
        std::lock_guard<std::mutex> lk(srv->mu);
        if (!form_batch(srv, batch, is_edit)) break;
        for (auto& r : batch) srv->scene_busy[r.req.scene_index]++;
        if (is_edit) srv->scene_edit_busy[batch[0].req.scene_index] = 1;
        srv->inflight++;
      }
      s.reqs.swap(batch);
      s.edit = is_edit;
      s.busy = true;
      s.start = srv->now();
      launch_batch(srv, s);
      any_busy = true;
    }
    if (srv->stop.load() && !any_busy) {
      std::lock_guard<std::mutex> lk(srv->mu);
      if (srv->queue.empty()) break;
    }
    if (any_busy) {
      std::this_thread::sleep_for(std::chrono::microseconds(10));
    } else {
      std::unique_lock<std::mutex> lk(srv->mu);
      srv->cv.wait_for(lk, std::chrono::milliseconds(2),
                       [&] { return !srv->queue.empty() || srv->stop.load(); });
    }
  }
}

}  // namespace
}  // namespace meso

using namespace meso;

extern "C" {

meso_status meso_server_create(meso_ctx* ctx, const meso_server_config* cfg, meso_scene* const* scenes,
                               uint32_t n_scenes, meso_server** out) {
  if (!ctx || !out || (n_scenes && !scenes)) return fail(MESO_ERR_INVALID_ARG, "server_create: null argument");
  if (n_scenes == 0) return fail(MESO_ERR_INVALID_ARG, "server_create: no scenes");
  meso_server* srv = new meso_server();
  srv->ctx = ctx;
  memset(&srv->cfg, 0, sizeof(srv->cfg));
  if (cfg) srv->cfg = *cfg;
  if (!srv->cfg.max_inflight_batches) srv->cfg.max_inflight_batches = 4;
  if (!srv->cfg.max_batch_requests) srv->cfg.max_batch_requests = kMaxBatch;
  if (!srv->cfg.max_batch_rays) srv->cfg.max_batch_rays = 16ull << 20;
  if (!srv->cfg.max_edit_quads) srv->cfg.max_edit_quads = 16ull << 20;
  const float* L = srv->cfg.light;
  if (L[0] == 0.0f && L[1] == 0.0f && L[2] == 0.0f) {
    // normalize(0.3, 0.5, 0.8) evaluated in double, then rounded
    const double n = std::sqrt(0.3 * 0.3 + 0.5 * 0.5 + 0.8 * 0.8);
    srv->light[0] = (float)(0.3 / n);
    srv->light[1] = (float)(0.5 / n);
    srv->light[2] = (float)(0.8 / n);
  } else {
    for (int a = 0; a < 3; a++) srv->light[a] = L[a];
  }
  uint32_t max_chunks = 0;
  for (uint32_t i = 0; i < n_scenes; i++) {
    if (!scenes[i]) {
      delete srv;
      return fail(MESO_ERR_INVALID_ARG, "server_create: null scene");
    }
    srv->scenes.push_back(scenes[i]);
    max_chunks = std::max<uint32_t>(max_chunks, (uint32_t)((scenes[i]->nx / 32) * (scenes[i]->ny / 32) *
                                                           (uint64_t)(scenes[i]->nz / 32)));
  }
  if (srv->cfg.keep_meshes) {
    for (uint32_t i = 0; i < n_scenes; i++) {
      meso_mesh_store* st = nullptr;
      const meso_status rc = meso_mesh_store_create(ctx, scenes[i], &st);
      if (rc != MESO_OK) {
        for (meso_mesh_store* t : srv->stores) meso_mesh_store_destroy(ctx, t);
        delete srv;
        return rc;
      }
      srv->stores.push_back(st);
    }
  }
  uint64_t store_bytes = 0;
  for (meso_mesh_store* t : srv->stores) store_bytes += store_device_bytes(t);
  srv->scene_busy.assign(n_scenes, 0);
  srv->scene_edit_busy.assign(n_scenes, 0);
  srv->dirty.assign(std::max<uint32_t>(max_chunks, 1), 0);
  // per slot: hits, view table, sums, quads, coordinates
  const uint32_t coord_cap = std::min<uint32_t>(max_chunks, MESO_MAX_CHUNKS_PER_CALL);
  const uint64_t per_slot = srv->cfg.max_batch_rays * sizeof(meso_hit) + raymarch_view_table_bytes(kMaxBatch) +
                            srv->cfg.max_edit_quads * 8 + 12ull * coord_cap + sizeof(unsigned long long) * kSums +
                            (srv->cfg.keep_meshes ? 16ull * coord_cap : 0);
  const uint64_t budget = srv->cfg.hbm_budget_bytes ? srv->cfg.hbm_budget_bytes : ctx->budget_bytes;
  const uint64_t scene_bytes = ctx->scene_bytes.load() + store_bytes;
  if (budget <= scene_bytes || per_slot > budget - scene_bytes) {
    for (meso_mesh_store* t : srv->stores) meso_mesh_store_destroy(ctx, t);
    delete srv;
    return fail(MESO_ERR_OVER_BUDGET, "server_create: HBM budget leaves no room for one batch slot");
  }
  const uint32_t fit = (uint32_t)std::min<uint64_t>((budget - scene_bytes) / per_slot, 64);
  const uint32_t n_slots = std::min<uint32_t>(srv->cfg.max_inflight_batches, fit);
  srv->slots.resize(n_slots);
  for (auto& s : srv->slots) {
    cudaError_t e = cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s.stream2, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s.forked, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s.joined, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMalloc(&s.d_hits, srv->cfg.max_batch_rays * sizeof(meso_hit));
    s.hit_cap = srv->cfg.max_batch_rays;
    s.table_bytes = raymarch_view_table_bytes(kMaxBatch);
    if (e == cudaSuccess) e = cudaMalloc(&s.d_table, s.table_bytes);
    if (e == cudaSuccess) e = cudaMalloc(&s.d_sums, sizeof(unsigned long long) * kSums);
    if (e == cudaSuccess) e = cudaMallocHost(&s.h_sums, sizeof(unsigned long long) * kSums);
    s.quad_cap = srv->cfg.max_edit_quads;
    if (e == cudaSuccess) e = cudaMalloc(&s.d_quads, s.quad_cap * 8);
    s.coord_cap = coord_cap;
    if (e == cudaSuccess) e = cudaMalloc(&s.d_coords, 12ull * std::max<uint32_t>(coord_cap, 1));
    if (e == cudaSuccess) e = cudaMallocHost(&s.h_coords, 12ull * std::max<uint32_t>(coord_cap, 1));
    if (e == cudaSuccess && srv->cfg.keep_hits) e = cudaMallocHost(&s.h_hits, srv->cfg.max_batch_rays * sizeof(meso_hit));
    if (e == cudaSuccess && srv->cfg.keep_meshes) {
      e = cudaMalloc(&s.d_counts, 4ull * std::max<uint32_t>(coord_cap, 1));
      if (e == cudaSuccess) e = cudaMalloc(&s.d_place, 12ull * std::max<uint32_t>(coord_cap, 1));
      if (e == cudaSuccess) e = cudaMallocHost(&s.h_flags, sizeof(unsigned long long));
      if (e == cudaSuccess) *s.h_flags = 0;
    }
    if (e != cudaSuccess) {
      for (auto& t : srv->slots) release_slot(t);
      for (meso_mesh_store* t : srv->stores) meso_mesh_store_destroy(ctx, t);
      delete srv;
      return cuda_fail(e, "server_create: slot allocation");
    }
  }
  srv->t0 = std::chrono::steady_clock::now();
  srv->th = std::thread(scheduler, srv);
  *out = srv;
  return MESO_OK;
}

meso_status meso_server_submit(meso_server* srv, const meso_request* req, uint64_t* request_id) {
  if (!srv || !req) return fail(MESO_ERR_INVALID_ARG, "server_submit: null argument");
  if (srv->stop.load()) return fail(MESO_ERR_SHUTDOWN, "server_submit: server is shutting down");
  if (req->scene_index >= srv->scenes.size()) return fail(MESO_ERR_INVALID_ARG, "server_submit: bad scene index");
  if (req->kind > MESO_REQ_EDIT_REMESH_RENDER) return fail(MESO_ERR_INVALID_ARG, "server_submit: bad kind");
  const meso_camera& c = req->camera;
  if (c.width == 0 || c.height == 0 || c.width > 16384 || c.height > 16384)
    return fail(MESO_ERR_INVALID_ARG, "server_submit: image size out of range");
  if (req->n_edits && !req->edits) return fail(MESO_ERR_INVALID_ARG, "server_submit: null edits");
  SrvRequest r;
  r.req = *req;
  r.req.edits = nullptr;
  if (req->kind == MESO_REQ_EDIT_REMESH_RENDER) r.edits.assign(req->edits, req->edits + req->n_edits);
  r.pixels = pixels_of(c);
  // a destination the raymarch kernel can store into directly (kept hits
  // are read from the batch buffer, so they keep every view there)
  if (req->dst_hits && !srv->cfg.keep_hits) {
    cudaPointerAttributes pa;
    if (cudaPointerGetAttributes(&pa, req->dst_hits) == cudaSuccess) {
      void* dp = nullptr;
      if ((pa.type == cudaMemoryTypeDevice || pa.type == cudaMemoryTypeManaged) && pa.device == srv->ctx->device)
        dp = pa.devicePointer;
      else if (pa.type == cudaMemoryTypeHost)
        dp = pa.devicePointer;
      if (dp && !(reinterpret_cast<uintptr_t>(dp) & 7u)) {
        r.d_dst = static_cast<meso_hit*>(dp);
        r.dst_host = pa.type == cudaMemoryTypeHost;
      }
    } else {
      cudaGetLastError();
    }
  }
  std::lock_guard<std::mutex> lk(srv->mu);
  r.id = srv->next_id++;
  r.submit = srv->now();
  if (request_id) *request_id = r.id;
  const bool too_big = srv->slots.empty() || r.pixels > srv->slots[0].hit_cap;
  const bool full = srv->cfg.max_queue && srv->queue.size() >= srv->cfg.max_queue;
  if (too_big || full) {
    srv->done.push_back(make_completion(srv, r, MESO_ERR_OVER_BUDGET, r.submit));
    return MESO_OK;
  }
  srv->queue.push_back(std::move(r));
  srv->cv.notify_all();
  return MESO_OK;
}

meso_status meso_server_poll(meso_server* srv, meso_completion* out, uint32_t max, uint32_t* n) {
  if (!srv || !n || (max && !out)) return fail(MESO_ERR_INVALID_ARG, "server_poll: null argument");
  std::lock_guard<std::mutex> lk(srv->mu);
  const uint32_t k = (uint32_t)std::min<size_t>(max, srv->done.size());
  for (uint32_t i = 0; i < k; i++) out[i] = srv->done[i];
  srv->done.erase(srv->done.begin(), srv->done.begin() + k);
  *n = k;
  return MESO_OK;
}

meso_status meso_server_fetch_hits(meso_server* srv, uint64_t id, meso_hit* h_hits, uint64_t capacity) {
  if (!srv || !h_hits) return fail(MESO_ERR_INVALID_ARG, "server_fetch_hits: null argument");
  std::lock_guard<std::mutex> lk(srv->mu);
  auto it = srv->kept.find(id);
  if (it == srv->kept.end()) return fail(MESO_ERR_NOT_READY, "server_fetch_hits: no kept hits for this request");
  if (it->second.size() > capacity) return fail(MESO_ERR_OVERFLOW, "server_fetch_hits: buffer too small");
  std::copy(it->second.begin(), it->second.end(), h_hits);
  srv->kept.erase(it);
  return MESO_OK;
}

meso_status meso_server_drain(meso_server* srv, double timeout_s) {
  if (!srv) return fail(MESO_ERR_INVALID_ARG, "server_drain: null server");
  std::unique_lock<std::mutex> lk(srv->mu);
  const bool ok = srv->cv.wait_for(lk, std::chrono::duration<double>(timeout_s),
                                   [&] { return srv->queue.empty() && srv->inflight == 0; });
  return ok ? MESO_OK : fail(MESO_ERR_TIMEOUT, "server_drain: requests still pending");
}

double meso_server_now(const meso_server* srv) { return srv ? srv->now() : 0.0; }

meso_status meso_server_destroy(meso_server* srv) {
  if (!srv) return MESO_OK;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->stop.store(true);
    srv->cv.notify_all();
  }
  if (srv->th.joinable()) srv->th.join();
  for (auto& s : srv->slots) release_slot(s);
  for (meso_mesh_store* t : srv->stores) meso_mesh_store_destroy(srv->ctx, t);
  delete srv;
  return MESO_OK;
}

meso_status meso_server_get_store(meso_server* srv, uint32_t scene_index, meso_mesh_store** out) {
  if (!srv || !out) return fail(MESO_ERR_INVALID_ARG, "server_get_store: null argument");
  if (srv->stores.empty()) return fail(MESO_ERR_INVALID_ARG, "server_get_store: the server keeps no meshes");
  if (scene_index >= srv->stores.size()) return fail(MESO_ERR_INVALID_ARG, "server_get_store: bad scene index");
  *out = srv->stores[scene_index];
  return MESO_OK;
}

}  // extern "C"
