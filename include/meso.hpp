// meso.hpp -- header-only C++ wrappers over the C ABI in meso.h, shaped like
// the reference's chunk-manager calls so a MesoEngine-style host can swap its
// generator/pool/draw path for device calls:
//   FChunkManage::Initialize (Runtimes/Voxel/Chunk/ChunkManager.h:90-102)  -> meso::Context
//   generator + FChunkPool::PushChunk (ChunkManager.h:183-210,
//     Runtimes/Voxel/Chunk/ChunkPool.h:623-628)                              -> meso::Scene
//   FChunkPool::PushToBlockPool (ChunkPool.h:381-445)                      -> meso::Scene::mesh
//   the imposter draw (Samples/SimpleVoxel.cpp:374-393)                    -> meso::Scene::render
//   chunk slots kept in the pools, replaced on regeneration
//     (ChunkPool.h:446-622, upload :653-679)                               -> meso::MeshStore
//   ThreadPool + TDoubleBufferQueue (Runtimes/Thread/ThreadPool.h:7-127,
//     Runtimes/Thread/DoubleBufferQueue.h:4-51)                            -> meso::Server
// Errors become meso::Error exceptions on the C++ side only; the C ABI below
// never throws.
#pragma once
#include <stdexcept>
#include <string>
#include <vector>

#include "meso.h"

namespace meso {

struct Error : std::runtime_error {
  meso_status status;
  Error(meso_status s, const std::string& what) : std::runtime_error(what), status(s) {}
};

inline void check(meso_status s) {
  if (s != MESO_OK) throw Error(s, std::string(meso_status_string(s)) + ": " + meso_last_error_string());
}

class Context {
 public:
  explicit Context(const meso_config& cfg = meso_config()) { check(meso_ctx_create(&cfg, &ctx_)); }
  ~Context() { meso_ctx_destroy(ctx_); }
  Context(const Context&) = delete;
  Context& operator=(const Context&) = delete;
  meso_ctx* get() const { return ctx_; }
  void sync(void* stream = nullptr) const { check(meso_sync(ctx_, stream)); }

 private:
  meso_ctx* ctx_ = nullptr;
};

class Scene {
 public:
  Scene(Context& ctx, const meso_terrain& t, uint64_t spare_bricks = 0) : ctx_(&ctx) {
    check(meso_scene_create_terrain(ctx.get(), &t, spare_bricks, &scene_));
  }
  Scene(Context& ctx, const std::vector<uint16_t>& grid, int32_t nx, int32_t ny, int32_t nz,
        uint64_t spare_bricks = 0)
      : ctx_(&ctx) {
    check(meso_scene_create_dense(ctx.get(), grid.data(), nx, ny, nz, spare_bricks, &scene_));
  }
  ~Scene() { meso_scene_destroy(ctx_->get(), scene_); }
  Scene(const Scene&) = delete;
  Scene& operator=(const Scene&) = delete;
  meso_scene* get() const { return scene_; }

  // Greedy quads of the chunks at device chunk coordinates d_coords (int32
  // triples); returns the quad count (throws MESO_ERR_OVERFLOW if it exceeds
  // out.capacity).
  uint64_t mesh(const int32_t* d_coords, uint32_t n, const meso_mesh_output& out, void* stream = nullptr) const {
    meso_mesh_source src{};
    src.kind = MESO_SRC_BRICKMAP;
    src.scene = scene_;
    check(meso_mesh_chunks(ctx_->get(), &src, d_coords, n, &out, stream));
    uint64_t count = 0;
    check(meso_mesh_check(ctx_->get(), &out, stream, &count));
    return count;
  }

  // One view, hits into device memory (width*height records).
  void render(const meso_camera& cam, const float light[3], meso_hit* d_hits, bool shadow = true,
              void* stream = nullptr) const {
    const meso_scene* s = scene_;
    check(meso_raymarch(ctx_->get(), &s, &cam, 1, light, shadow ? MESO_RAY_SHADOW : 0u, d_hits, stream));
  }

  // Sphere edits; returns the sorted linear indices of the dirty 32^3 chunks.
  std::vector<uint32_t> edit(const std::vector<meso_sphere_edit>& spheres, void* stream = nullptr) {
    const meso_scene_info info = this->info();
    std::vector<uint32_t> dirty((size_t)(info.nx / 32) * (info.ny / 32) * (info.nz / 32));
    uint32_t n = 0;
    check(meso_edit_spheres(ctx_->get(), scene_, spheres.data(), (uint32_t)spheres.size(), dirty.data(),
                            (uint32_t)dirty.size(), &n, stream));
    dirty.resize(n);
    return dirty;
  }

  meso_scene_info info() const {
    meso_scene_info i{};
    check(meso_scene_get_info(ctx_->get(), scene_, &i));
    return i;
  }

 private:
  Context* ctx_;
  meso_scene* scene_ = nullptr;
};

// A scene's quads kept on the device: one arena plus a segment per chunk.
class MeshStore {
 public:
  MeshStore(Context& ctx, const Scene& scene) : ctx_(&ctx) { check(meso_mesh_store_create(ctx.get(), scene.get(), &store_)); }
  ~MeshStore() { meso_mesh_store_destroy(ctx_->get(), store_); }
  MeshStore(const MeshStore&) = delete;
  MeshStore& operator=(const MeshStore&) = delete;
  meso_mesh_store* get() const { return store_; }

  // Remeshes the chunks (linear chunk indices, e.g. Scene::edit's result)
  // and replaces their segments.
  void update(const std::vector<uint32_t>& chunks) {
    check(meso_mesh_store_update(ctx_->get(), store_, chunks.data(), (uint32_t)chunks.size()));
  }
  // The chunks' quads into d_out (capacity quads); returns their count.
  uint64_t gather(const std::vector<uint32_t>& chunks, uint64_t* d_out, uint64_t capacity) const {
    uint64_t total = 0;
    check(meso_mesh_store_gather(ctx_->get(), store_, chunks.data(), (uint32_t)chunks.size(), d_out, capacity,
                                 &total));
    return total;
  }
  meso_mesh_store_info info() const {
    meso_mesh_store_info i{};
    check(meso_mesh_store_get_info(ctx_->get(), store_, &i));
    return i;
  }

 private:
  Context* ctx_;
  meso_mesh_store* store_ = nullptr;
};

// The serving loop over resident scenes: submit requests from any thread,
// poll their completions.
class Server {
 public:
  Server(Context& ctx, const std::vector<meso_scene*>& scenes, const meso_server_config& cfg = meso_server_config()) {
    check(meso_server_create(ctx.get(), &cfg, scenes.data(), (uint32_t)scenes.size(), &srv_));
  }
  ~Server() { meso_server_destroy(srv_); }
  Server(const Server&) = delete;
  Server& operator=(const Server&) = delete;
  meso_server* get() const { return srv_; }

  uint64_t submit(const meso_request& req) {
    uint64_t id = 0;
    check(meso_server_submit(srv_, &req, &id));
    return id;
  }
  std::vector<meso_completion> poll(uint32_t max = 1024) {
    std::vector<meso_completion> out(max);
    uint32_t n = 0;
    check(meso_server_poll(srv_, out.data(), max, &n));
    out.resize(n);
    return out;
  }
  void drain(double timeout_s = 60.0) { check(meso_server_drain(srv_, timeout_s)); }

 private:
  meso_server* srv_ = nullptr;
};

}  // namespace meso
