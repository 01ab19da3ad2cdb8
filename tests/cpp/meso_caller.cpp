// A compiled C++ caller of mesoengine_gb300, built against include/meso.hpp
// and libmeso_gb300.so the way a MesoEngine-style host would link it.  It
// builds the 128^3 golden terrain, renders the golden 96x64 view and compares
// the hits byte for byte with the golden file, meshes every chunk of the
// scene, serves the golden view through the request loop (hits delivered
// into page-locked host memory and into device memory, both compared byte
// for byte), applies sphere edits and keeps a mesh store current, and
// writes the quads it got (sorted) for the test to compare with the oracle.
//
//   meso_caller <camera.bin> <golden_hits.bin> <out_dir>
// camera.bin: one meso_camera (72 bytes); golden_hits.bin: 96*64 meso_hit.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iterator>
#include <vector>

#include "meso.hpp"

static std::vector<char> read_file(const char* path) {
  std::ifstream f(path, std::ios::binary);
  return std::vector<char>(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
}

template <typename T>
static void write_file(const std::string& path, const std::vector<T>& v) {
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char*>(v.data()), (std::streamsize)(v.size() * sizeof(T)));
}

// Device buffer owned through the C ABI helpers.
struct DevBuf {
  meso_ctx* ctx;
  void* p = nullptr;
  DevBuf(meso::Context& c, size_t bytes) : ctx(c.get()) { meso::check(meso_dev_alloc(ctx, bytes, &p)); }
  ~DevBuf() { meso_dev_free(ctx, p); }
};

int main(int argc, char** argv) {
  if (argc != 4) {
    std::fprintf(stderr, "usage: meso_caller camera.bin golden_hits.bin out_dir\n");
    return 2;
  }
  try {
    meso::Context ctx;
    const meso_terrain t{128, 128, 128, 2, 64, 6, 7.0f, 32.0f, 48, 0.7f};
    meso::Scene scene(ctx, t, /*spare_bricks=*/8192);
    const meso_scene_info info = scene.info();
    if (info.n_bricks != 720) {
      std::fprintf(stderr, "terrain: %llu bricks, expected 720\n", (unsigned long long)info.n_bricks);
      return 1;
    }
    // render the golden view
    const std::vector<char> cam_bytes = read_file(argv[1]);
    const std::vector<char> golden = read_file(argv[2]);
    if (cam_bytes.size() != sizeof(meso_camera) || golden.size() != 96 * 64 * sizeof(meso_hit)) {
      std::fprintf(stderr, "bad input files\n");
      return 2;
    }
    meso_camera cam;
    std::memcpy(&cam, cam_bytes.data(), sizeof(cam));
    const float light[3] = {0.30304575f, 0.50507629f, 0.80812204f};  // normalize(0.3, 0.5, 0.8)
    DevBuf d_hits(ctx, golden.size());
    scene.render(cam, light, static_cast<meso_hit*>(d_hits.p));
    std::vector<char> hits(golden.size());
    meso::check(meso_memcpy_d2h(ctx.get(), hits.data(), d_hits.p, hits.size(), nullptr));
    ctx.sync();
    if (hits != golden) {
      std::fprintf(stderr, "hits differ from the golden file\n");
      return 1;
    }
    // mesh all 4x4x4 chunks through the wrapper
    std::vector<int32_t> coords;
    for (int z = 0; z < 4; z++)
      for (int y = 0; y < 4; y++)
        for (int x = 0; x < 4; x++) coords.insert(coords.end(), {x, y, z});
    DevBuf d_coords(ctx, coords.size() * 4);
    meso::check(meso_memcpy_h2d(ctx.get(), d_coords.p, coords.data(), coords.size() * 4, nullptr));
    const uint64_t cap = 64 * 16384;
    DevBuf d_quads(ctx, cap * 8), d_count(ctx, 8);
    meso_mesh_output out{static_cast<uint64_t*>(d_quads.p), cap, static_cast<uint64_t*>(d_count.p), nullptr};
    const uint64_t nq = scene.mesh(static_cast<const int32_t*>(d_coords.p), 64, out);
    std::vector<uint64_t> quads(nq);
    meso::check(meso_memcpy_d2h(ctx.get(), quads.data(), d_quads.p, nq * 8, nullptr));
    ctx.sync();
    std::sort(quads.begin(), quads.end());
    write_file(std::string(argv[3]) + "/quads_before.bin", quads);
    // the golden view served: one request delivered into page-locked host
    // memory, one into device memory, both compared with the golden hits
    {
      meso::Server srv(ctx, {scene.get()});
      void* h_dst = nullptr;
      meso::check(meso_host_alloc_pinned(ctx.get(), golden.size(), &h_dst));
      DevBuf d_dst(ctx, golden.size());
      meso_request req{};
      req.kind = MESO_REQ_RENDER;
      req.scene_index = 0;
      req.camera = cam;
      req.flags = MESO_RAY_SHADOW;
      req.dst_hits = static_cast<meso_hit*>(h_dst);
      const uint64_t id_host = srv.submit(req);
      req.dst_hits = static_cast<meso_hit*>(d_dst.p);
      const uint64_t id_dev = srv.submit(req);
      srv.drain();
      const std::vector<meso_completion> done = srv.poll();
      bool seen_host = false, seen_dev = false;
      for (const meso_completion& c : done) {
        if (c.status != MESO_OK) {
          std::fprintf(stderr, "served request %llu failed: %d\n", (unsigned long long)c.request_id, c.status);
          return 1;
        }
        seen_host = seen_host || c.request_id == id_host;
        seen_dev = seen_dev || c.request_id == id_dev;
      }
      std::vector<char> served(golden.size());
      meso::check(meso_memcpy_d2h(ctx.get(), served.data(), d_dst.p, served.size(), nullptr));
      ctx.sync();
      const bool host_ok = std::memcmp(h_dst, golden.data(), golden.size()) == 0;
      meso::check(meso_host_free_pinned(ctx.get(), h_dst));
      if (!seen_host || !seen_dev || !host_ok || served != golden) {
        std::fprintf(stderr, "served hits differ from the golden file\n");
        return 1;
      }
    }
    // edits, then the resident mesh store brought up to date
    meso::MeshStore store(ctx, scene);
    std::vector<meso_sphere_edit> spheres;
    for (int k = 0; k < 12; k++) {
      meso_sphere_edit e{};
      e.center[0] = 11 * k % 128;
      e.center[1] = 37 * k % 128;
      e.center[2] = 5 + 3 * k;
      e.radius = 3 + k % 7;
      e.material = (uint16_t)(k % 3 == 0 ? 0 : 100 + 977 * k);
      spheres.push_back(e);
    }
    const std::vector<uint32_t> dirty = scene.edit(spheres);
    store.update(dirty);
    std::vector<uint32_t> all(64);
    for (uint32_t c = 0; c < 64; c++) all[c] = c;
    DevBuf d_all(ctx, cap * 8);
    const uint64_t total = store.gather(all, static_cast<uint64_t*>(d_all.p), cap);
    if (store.info().live_quads != total) {
      std::fprintf(stderr, "store holds %llu quads, gathered %llu\n", (unsigned long long)store.info().live_quads,
                   (unsigned long long)total);
      return 1;
    }
    std::vector<uint64_t> after(total);
    meso::check(meso_memcpy_d2h(ctx.get(), after.data(), d_all.p, total * 8, nullptr));
    ctx.sync();
    std::sort(after.begin(), after.end());
    write_file(std::string(argv[3]) + "/quads_after.bin", after);
    std::printf("ok: %llu quads, %zu dirty chunks, %llu quads after the edits\n", (unsigned long long)nq, dirty.size(),
                (unsigned long long)total);
    return 0;
  } catch (const meso::Error& e) {
    std::fprintf(stderr, "meso error: %s\n", e.what());
    return 1;
  }
}
