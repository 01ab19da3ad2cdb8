// meso_internal.h -- shared internals of the mesoengine_gb300 library:
// context/scene structs, error plumbing, sm_103a PTX wrappers (mbarrier,
// bulk and tensor TMA copies) and the bit-exact FP32 noise used by the
// device scene generators.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/meso.h"

// ------------------------------------------------------------------ errors

namespace meso {

void set_error(const std::string& msg);
meso_status fail(meso_status s, const std::string& msg);
meso_status cuda_fail(cudaError_t e, const char* what);

#define MESO_CUDA_TRY(expr)                                  \
  do {                                                       \
    cudaError_t _e = (expr);                                 \
    if (_e != cudaSuccess) return ::meso::cuda_fail(_e, #expr); \
  } while (0)

#define MESO_TRY(expr)                 \
  do {                                 \
    meso_status _s = (expr);           \
    if (_s != MESO_OK) return _s;      \
  } while (0)

// Device-side error flag bits (ctx->d_err).
enum : uint32_t {
  ERR_TIMEOUT = 1u,       // a bounded mbarrier wait gave up
  ERR_POOL_FULL = 2u,     // brick pool exhausted during an edit
  ERR_BAD_INPUT = 4u,     // out-of-range chunk coordinate
};

struct Tuning {
  uint32_t mesh_ctas_per_sm = 0;  // 0: two 16-warp CTAs per SM
  uint32_t mesh_chunks_per_ticket = 1;
  uint32_t ray_tile_w = 8;  // lanes of one warp along x
  uint32_t ray_warps_per_cta = 4;
};

}  // namespace meso

struct meso_ctx {
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;  // default stream of the context
  meso::Tuning tuning;
  uint64_t budget_bytes = 0;
  std::atomic<uint64_t> scene_bytes{0};
  std::atomic<uint64_t> launches{0};
  // small device scratch: [0] spare, [1] error flags, [2..63] spare
  uint32_t* d_scratch = nullptr;  // 16 words: [1] device error flags, [2] sink of the L2 probe
  // ring of queue tickets for persistent mesh launches; consecutive launches
  // take consecutive counters, so up to kTicketRing launches may overlap on
  // different streams
  static constexpr uint32_t kTicketRing = 64;
  uint32_t* d_tickets = nullptr;
  std::atomic<uint32_t> next_ticket{0};
  std::mutex mu;
};

struct meso_scene {
  int32_t nx = 0, ny = 0, nz = 0;
  int32_t bx = 0, by = 0, bz = 0;
  uint32_t* d_ptr = nullptr;   // brick pointers
  uint64_t* d_occ = nullptr;   // 8 words per slot
  uint16_t* d_mat = nullptr;   // 512 per slot
  // one byte per 4x4x4-brick cell (a 32^3 chunk): nonzero iff a brick of the
  // cell is occupied; lets a ray cross an empty cell in one jump
  uint8_t* d_macro = nullptr;
  // one byte per 16x16x16-brick cell (128^3 voxels, partial at the far
  // edges): nonzero iff one of its 32^3 cells is, or it extends past the grid
  uint8_t* d_macro2 = nullptr;
  // one byte per 64x64x64-brick cell (512^3 voxels), built like d_macro2 from it
  uint8_t* d_macro3 = nullptr;
  uint64_t capacity = 0;       // pool slots
  // allocator state (device): [0] bump (slots ever used), [1] free-stack top
  int64_t* d_alloc = nullptr;
  uint32_t* d_free = nullptr;  // free stack, capacity entries
  uint64_t bytes = 0;
  uint64_t live_bricks_host = 0;  // as of the last build/edit sync
};

namespace meso {

inline uint64_t n_bricks_of(const meso_scene* s) {
  return (uint64_t)s->bx * (uint64_t)s->by * (uint64_t)s->bz;
}
inline uint64_t n_macro_of(const meso_scene* s) { return n_bricks_of(s) / 64; }
inline uint64_t n_macro2_of(const meso_scene* s) {
  return (uint64_t)((s->bx + 15) / 16) * (uint64_t)((s->by + 15) / 16) * (uint64_t)((s->bz + 15) / 16);
}
inline uint64_t n_macro3_of(const meso_scene* s) {
  return (uint64_t)((s->bx + 63) / 64) * (uint64_t)((s->by + 63) / 64) * (uint64_t)((s->bz + 63) / 64);
}

inline cudaStream_t pick_stream(meso_ctx* ctx, void* s) {
  return s ? (cudaStream_t)s : ctx->stream;
}

// Scene-layer helpers shared by the edit and serving code.
meso_status scene_alloc(meso_ctx* ctx, int32_t nx, int32_t ny, int32_t nz, uint64_t capacity,
                        meso_scene** out);
void scene_release(meso_ctx* ctx, meso_scene* s);
// Recomputes the macro-cell map of a scene from its pointer grid: all cells,
// or the n cells listed in d_cells (linear macro-cell indices).
// Recomputes the cell maps: every cell (lists null), or the listed cells of
// 4^3, 16^3 and 64^3 bricks (each list sorted unique, children before parents).
meso_status rebuild_macro(meso_ctx* ctx, meso_scene* s, const uint32_t* d_cells, uint32_t n, cudaStream_t st,
                          const uint32_t* d_cells2 = nullptr, uint32_t n2 = 0, const uint32_t* d_cells3 = nullptr,
                          uint32_t n3 = 0);

// Kernel launchers (defined in the .cu files).
// chunk_id_base: added to the list index in each quad's chunk field (the
// chunks are entries chunk_id_base .. of a longer list); accumulate: the
// output count is not zeroed first, so several launches append to one buffer.
meso_status launch_mesh(meso_ctx* ctx, const meso_mesh_source* src, const int32_t* d_coords,
                        uint32_t n_chunks, const meso_mesh_output* out, cudaStream_t st, bool per_launch,
                        uint32_t chunk_id_base = 0, bool accumulate = false);
struct RayView;
// view_out (optional, n_views entries): where view v's hits go, a device or
// device-mapped address aligned to 8 bytes; a null entry (or a null array)
// keeps the view's place in d_hits (views packed in order).  d_hash
// (optional; at most kRayHashViews views, not with d_stats): the kernel adds
// view v's order-sensitive hit checksum into the kRayHashSlots partial sums
// d_hash[v * kRayHashSlots + s] and its traced shadow rays into
// d_hash[kRayHashShadow + v * kRayHashSlots + s] (s = the CTA's index mod
// kRayHashSlots, so that the warps' atomics spread over several addresses);
// the caller adds the partial sums.  host_out: some output is page-locked
// host memory, so the kernel writes whole rows of a CTA's pixels.
constexpr uint32_t kRayHashViews = 64, kRayHashSlots = 8;
constexpr uint32_t kRayHashShadow = kRayHashViews * kRayHashSlots;  // first shadow entry
constexpr uint32_t kRayHashEntries = 2 * kRayHashShadow;
meso_status launch_raymarch(meso_ctx* ctx, const meso_scene* const* scenes, const meso_camera* cams,
                            uint32_t n_views, const float light[3], uint32_t flags, meso_hit* d_hits,
                            cudaStream_t st, void* d_view_table, size_t view_table_bytes,
                            uint64_t* d_stats = nullptr, meso_hit* const* view_out = nullptr,
                            unsigned long long* d_hash = nullptr, bool host_out = false);
size_t raymarch_view_table_bytes(uint32_t n_views);

// Mesh store internals shared with the serving loop (store.cu).
// Places the quads of the n chunks at d_coords that a batched mesh launch
// left in d_temp (counts per chunk in d_counts) into the store's segments;
// stream-ordered.  d_work holds 12 * n bytes.
meso_status store_place_async(meso_ctx* ctx, meso_mesh_store* S, const int32_t* d_coords, uint32_t n,
                              const uint64_t* d_temp, uint64_t temp_cap, const unsigned long long* d_temp_count,
                              const uint32_t* d_counts, void* d_work, cudaStream_t st);
// Remeshes the listed chunks (linear indices) and waits until the store holds them.
meso_status store_update_sync(meso_ctx* ctx, meso_mesh_store* S, const uint32_t* h_chunks, uint32_t n,
                              cudaStream_t st);
// Device word of the store's flags (nonzero: a placement failed and the
// chunks of that update must be placed again with store_update_sync).
unsigned long long* store_flags_word(meso_mesh_store* S);
uint64_t store_device_bytes(const meso_mesh_store* S);

}  // namespace meso

// ------------------------------------------------------------ PTX wrappers

#ifdef __CUDACC__
namespace meso {
namespace dev {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Makes generic-proxy shared-memory state (barrier init, prior reads and
// writes) ordered before subsequent async-proxy (TMA) accesses.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ uint64_t global_timer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait on an mbarrier phase.  Returns false after limit_ns.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint64_t limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  uint64_t t0 = global_timer_ns();
  for (;;) {
    if (mbar_try_wait(bar, parity)) return true;
    if (global_timer_ns() - t0 > limit_ns) return false;
  }
}

// 1-D bulk copy global -> shared, completion counted on bar (bytes % 16 == 0,
// both addresses 16-byte aligned).
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// 3-D tiled tensor copy global -> shared (x * element size must be a multiple of 16).
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int32_t x, int32_t y, int32_t z,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
      "%4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// L2 prefetch of a global range (address 16-byte aligned, bytes % 16 == 0).
__device__ __forceinline__ void bulk_prefetch_l2(const void* src, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

// L2 prefetch of one box of a 3-D tiled tensor map.
__device__ __forceinline__ void tma_prefetch_3d(const CUtensorMap* map, int32_t x, int32_t y, int32_t z) {
  asm volatile("cp.async.bulk.prefetch.tensor.3d.L2.global.tile [%0, {%1, %2, %3}];" ::"l"(map), "r"(x), "r"(y),
               "r"(z)
               : "memory");
}

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// ---------------------------------------------------------------- noise
// pcg3d (Jarzynski & Olano 2020), third lane.
__device__ __forceinline__ uint32_t pcg3d(uint32_t x, uint32_t y, uint32_t z) {
  x = x * 1664525u + 1013904223u;
  y = y * 1664525u + 1013904223u;
  z = z * 1664525u + 1013904223u;
  x += y * z;
  y += z * x;
  z += x * y;
  x ^= x >> 16;
  y ^= y >> 16;
  z ^= z >> 16;
  x += y * z;
  y += z * x;
  z += x * y;
  return z;
}

__device__ __forceinline__ float lattice(uint32_t ix, uint32_t iy, uint32_t iz, uint32_t seed) {
  uint32_t h = pcg3d(ix + seed * 0x9E3779B9u, iy ^ (seed * 0x85EBCA6Bu), iz + seed * 0xC2B2AE35u);
  return __fmul_rn((float)(h >> 8), 1.0f / 16777216.0f);
}

// Every FP32 operation below is a single correctly rounded IEEE operation in
// a fixed order, so host code compiled without contraction reproduces it.
__device__ __forceinline__ float fade(float t) {
  float a = __fmul_rn(t, 6.0f);
  a = __fsub_rn(a, 15.0f);
  a = __fmul_rn(t, a);
  a = __fadd_rn(a, 10.0f);
  float b = __fmul_rn(t, t);
  b = __fmul_rn(b, t);
  return __fmul_rn(b, a);
}

__device__ __forceinline__ float lerp_rn(float a, float b, float t) {
  float d = __fsub_rn(b, a);
  d = __fmul_rn(d, t);
  return __fadd_rn(a, d);
}

__device__ __forceinline__ float cell_frac(uint32_t p, uint32_t period) {
  float f = __uint2float_rn(p % period);
  f = __fadd_rn(f, 0.5f);
  return __fdiv_rn(f, __uint2float_rn(period));
}

__device__ __forceinline__ float vnoise3(uint32_t x, uint32_t y, uint32_t z, uint32_t period, uint32_t seed) {
  uint32_t ix = x / period, iy = y / period, iz = z / period;
  float sx = fade(cell_frac(x, period));
  float sy = fade(cell_frac(y, period));
  float sz = fade(cell_frac(z, period));
  float c000 = lattice(ix, iy, iz, seed), c100 = lattice(ix + 1, iy, iz, seed);
  float c010 = lattice(ix, iy + 1, iz, seed), c110 = lattice(ix + 1, iy + 1, iz, seed);
  float c001 = lattice(ix, iy, iz + 1, seed), c101 = lattice(ix + 1, iy, iz + 1, seed);
  float c011 = lattice(ix, iy + 1, iz + 1, seed), c111 = lattice(ix + 1, iy + 1, iz + 1, seed);
  float x00 = lerp_rn(c000, c100, sx), x10 = lerp_rn(c010, c110, sx);
  float x01 = lerp_rn(c001, c101, sx), x11 = lerp_rn(c011, c111, sx);
  float y0 = lerp_rn(x00, x10, sy), y1 = lerp_rn(x01, x11, sy);
  return lerp_rn(y0, y1, sz);
}

__device__ __forceinline__ float vnoise2(uint32_t x, uint32_t y, uint32_t period, uint32_t seed) {
  uint32_t ix = x / period, iy = y / period;
  const uint32_t iz = 0x5BD1E995u;
  float sx = fade(cell_frac(x, period));
  float sy = fade(cell_frac(y, period));
  float c00 = lattice(ix, iy, iz, seed), c10 = lattice(ix + 1, iy, iz, seed);
  float c01 = lattice(ix, iy + 1, iz, seed), c11 = lattice(ix + 1, iy + 1, iz, seed);
  float x0 = lerp_rn(c00, c10, sx), x1 = lerp_rn(c01, c11, sx);
  return lerp_rn(x0, x1, sy);
}

__device__ __forceinline__ float fbm2(uint32_t x, uint32_t y, uint32_t period, int octaves, uint32_t seed) {
  float sum = 0.0f, amp = 1.0f, norm = 0.0f;
  for (int o = 0; o < octaves; o++) {
    uint32_t p = period >> o;
    if (p == 0) p = 1;
    float n = vnoise2(x, y, p, seed + (uint32_t)o);
    n = __fmul_rn(amp, n);
    sum = __fadd_rn(sum, n);
    norm = __fadd_rn(norm, amp);
    amp = __fmul_rn(amp, 0.5f);
  }
  return __fdiv_rn(sum, norm);
}

}  // namespace dev
}  // namespace meso
#endif  // __CUDACC__
