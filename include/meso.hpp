// meso.hpp -- header-only C++ wrappers over the C ABI in meso.h, shaped like
// the reference's chunk-manager calls so a MesoEngine-style host can swap its
// generator/pool/draw path for device calls:
//   FChunkManage::Initialize (Runtimes/Voxel/Chunk/ChunkManager.h:90-102)  -> meso::Context
//   generator + FChunkPool::PushChunk (ChunkManager.h:183-210,
//     Runtimes/Voxel/Chunk/ChunkPool.h:623-628)                              -> meso::Scene
//   FChunkPool::PushToBlockPool (ChunkPool.h:381-445)                      -> meso::Scene::mesh
//   the imposter draw (Samples/SimpleVoxel.cpp:374-393)                    -> meso::Scene::render
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

}  // namespace meso
