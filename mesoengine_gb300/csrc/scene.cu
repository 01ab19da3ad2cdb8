// scene.cu -- device-resident brick-map scenes: build from the seeded terrain
// generator or from a dense grid, the dense/chunk generators of the meshing
// workloads, and sphere edits with a device brick allocator.
//
// The reference keeps chunks as host vectors of blocks in ring-buffer pools
// with importance eviction (Runtimes/Voxel/Chunk/ChunkPool.h:83-181,
// :446-622) and regenerates them from a sin-hash SDF on host threads
// (Runtimes/Helper/GeneratorHelper.h:120-150).  Here a scene is three device
// arrays: a pointer grid (one uint32 per 8^3 brick, all-ones = empty, the
// reference's INT_MAX-sentinel idea, Runtimes/Voxel/Block/Block.h:16-18), a
// pool of 64-byte occupancy masks (word z, bit x+8y; the FVolume 8^3 bitmask of
// Runtimes/Voxel/VoxelStructure.h:30-39) and a pool of 1 KiB uint16 material
// bricks.  Bricks are numbered in pointer-grid order by an exclusive scan, so
// a build is deterministic.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <set>
#include <vector>

#include "meso_internal.h"

namespace meso {
namespace {

using namespace ::meso::dev;

constexpr uint32_t kFull = 0xFFFFFFFFu;

struct TerrainDev {
  int32_t nx, ny, nz;
  uint32_t seed, height_period;
  int32_t height_octaves;
  float height_base, height_amp;
  uint32_t cave_period;
  float cave_threshold;
};

TerrainDev to_dev(const meso_terrain& t) {
  TerrainDev d;
  d.nx = t.nx;
  d.ny = t.ny;
  d.nz = t.nz;
  d.seed = t.seed;
  d.height_period = t.height_period;
  d.height_octaves = t.height_octaves;
  d.height_base = t.height_base;
  d.height_amp = t.height_amp;
  d.cave_period = t.cave_period;
  d.cave_threshold = t.cave_threshold;
  return d;
}

__device__ __forceinline__ uint16_t terrain_voxel(const TerrainDev& T, float h, uint32_t x, uint32_t y, uint32_t z) {
  if (!(__uint2float_rn(z) < h)) return 0;
  const float c = vnoise3(x, y, z, T.cave_period, T.seed + 100u);
  if (c > T.cave_threshold) return 0;
  const int depth = (int)floorf(h) - (int)z;
  return (uint16_t)(1 + ((depth >> 2) & 63));
}

__global__ void heights_kernel(TerrainDev T, float* heights) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= (uint64_t)T.nx * T.ny) return;
  const uint32_t x = (uint32_t)(i % T.nx), y = (uint32_t)(i / T.nx);
  const float f = fbm2(x, y, T.height_period, T.height_octaves, T.seed);
  heights[i] = __fadd_rn(T.height_base, __fmul_rn(T.height_amp, f));
}

__global__ void column_max_kernel(TerrainDev T, const float* heights, float* hmax) {
  const int bx = T.nx / 8, by = T.ny / 8;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= bx * by) return;
  const int X = (i % bx) * 8, Y = (i / bx) * 8;
  float m = -__builtin_huge_valf();
  for (int ly = 0; ly < 8; ly++)
    for (int lx = 0; lx < 8; lx++) m = fmaxf(m, heights[(size_t)(Y + ly) * T.nx + X + lx]);
  hmax[i] = m;
}

// One warp per brick; lane covers voxels lane + 32k (x = i&7, y = (i>>3)&7, z = i>>6).
template <bool kFill>
__global__ void terrain_brick_kernel(TerrainDev T, const float* heights, const float* hmax, uint8_t* flags,
                                     const uint32_t* ptr, uint64_t* occ, uint16_t* mat) {
  const int bx = T.nx / 8, by = T.ny / 8, bz = T.nz / 8;
  const uint64_t nb = (uint64_t)bx * by * bz;
  const int lane = threadIdx.x & 31;
  const uint64_t wstride = (uint64_t)gridDim.x * (blockDim.x >> 5);
  for (uint64_t b = blockIdx.x * (uint64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); b < nb; b += wstride) {
    const int X = (int)(b % bx), Y = (int)((b / bx) % by), Z = (int)(b / ((uint64_t)bx * by));
    if (kFill) {
      if (!flags[b]) continue;
    } else {
      if (!((float)(Z * 8) < hmax[(size_t)Y * bx + X])) {
        if (lane == 0) flags[b] = 0;
        continue;
      }
    }
    const uint32_t slot = kFill ? ptr[b] : 0u;
    bool any = false;
    for (int k = 0; k < 16; k++) {
      const int i = lane + 32 * k;
      const uint32_t x = X * 8 + (i & 7), y = Y * 8 + ((i >> 3) & 7), z = Z * 8 + (i >> 6);
      const float h = heights[(size_t)y * T.nx + x];
      const uint16_t m = terrain_voxel(T, h, x, y, z);
      if (kFill) {
        mat[(size_t)slot * 512 + i] = m;
        // voxel i = lane + 32k is bit (i mod 32) of 32-bit word k of the
        // brick's occupancy (word z of 64 bits = 32-bit words 2z, 2z+1)
        const uint32_t bits = __ballot_sync(kFull, m != 0);
        if (lane == 0) reinterpret_cast<uint32_t*>(occ + (size_t)slot * 8)[k] = bits;
      } else {
        any |= m != 0;
      }
    }
    if (!kFill) {
      const bool f = __any_sync(kFull, any);
      if (lane == 0) flags[b] = f ? 1 : 0;
    }
  }
}

// ---------------------------------------------------------------- scan
constexpr int kScanThreads = 1024;
constexpr int kScanPer = 4;
constexpr int kScanTile = kScanThreads * kScanPer;

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* warp_sums, uint32_t& total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(kFull, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t s = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0u;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(kFull, s, o);
      if (lane >= o) s += y;
    }
    warp_sums[lane] = s;  // inclusive
  }
  __syncthreads();
  const uint32_t before = warp ? warp_sums[warp - 1] : 0u;
  total = warp_sums[(blockDim.x >> 5) - 1];
  __syncthreads();
  return before + x - v;
}

// flags (uint8) -> out (exclusive prefix within tile), tile sums.
__global__ void scan_tiles_kernel(const uint8_t* flags, uint64_t n, uint32_t* out, uint32_t* tile_sums) {
  __shared__ uint32_t ws[32];
  const uint64_t base = blockIdx.x * (uint64_t)kScanTile + threadIdx.x * (uint64_t)kScanPer;
  uint32_t v[kScanPer], s = 0;
  for (int k = 0; k < kScanPer; k++) {
    v[k] = (base + k < n) ? flags[base + k] : 0u;
    s += v[k];
  }
  uint32_t total;
  uint32_t ex = block_exclusive_scan(s, ws, total);
  for (int k = 0; k < kScanPer; k++) {
    if (base + k < n) out[base + k] = ex;
    ex += v[k];
  }
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

// single block: exclusive scan of tile sums in place; grand total to *total.
__global__ void scan_sums_kernel(uint32_t* sums, uint32_t n, uint32_t* total) {
  __shared__ uint32_t ws[32];
  uint32_t carry = 0;
  for (uint32_t base = 0; base < n; base += kScanThreads) {
    const uint32_t i = base + threadIdx.x;
    const uint32_t v = i < n ? sums[i] : 0u;
    uint32_t t;
    const uint32_t ex = block_exclusive_scan(v, ws, t);
    if (i < n) sums[i] = carry + ex;
    carry += t;
  }
  if (threadIdx.x == 0) *total = carry;
}

// ptr[b] = flags[b] ? tile offset + local : EMPTY
__global__ void scan_finish_kernel(const uint8_t* flags, uint64_t n, const uint32_t* tile_sums, uint32_t* ptr) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  ptr[i] = flags[i] ? ptr[i] + tile_sums[i / kScanTile] : MESO_EMPTY_BRICK;
}

// Numbers bricks flagged nonzero in pointer-grid order.  Returns the count.
meso_status number_bricks(meso_ctx* ctx, const uint8_t* d_flags, uint64_t nb, uint32_t* d_ptr, cudaStream_t st,
                          uint64_t* count) {
  const uint64_t tiles = (nb + kScanTile - 1) / kScanTile;
  if (tiles > 0xFFFFFFFFull) return fail(MESO_ERR_INVALID_ARG, "scene too large");
  uint32_t* d_sums = nullptr;
  MESO_CUDA_TRY(cudaMallocAsync(&d_sums, sizeof(uint32_t) * (tiles + 1), st));
  scan_tiles_kernel<<<(unsigned)tiles, kScanThreads, 0, st>>>(d_flags, nb, d_ptr, d_sums);
  scan_sums_kernel<<<1, kScanThreads, 0, st>>>(d_sums, (uint32_t)tiles, d_sums + tiles);
  scan_finish_kernel<<<(unsigned)((nb + 255) / 256), 256, 0, st>>>(d_flags, nb, d_sums, d_ptr);
  ctx->launches.fetch_add(3);
  uint32_t h_total = 0;
  MESO_CUDA_TRY(cudaMemcpyAsync(&h_total, d_sums + tiles, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  MESO_CUDA_TRY(cudaFreeAsync(d_sums, st));
  MESO_CUDA_TRY(cudaStreamSynchronize(st));
  MESO_CUDA_TRY(cudaGetLastError());
  *count = h_total;
  return MESO_OK;
}

// ---------------------------------------------------------- dense -> bricks
// T: uint16_t or uint8_t materials of a dense grid (x fastest).
template <typename T>
__global__ void dense_flag_kernel(const T* grid, int nx, int ny, int nz, uint8_t* flags) {
  const int bx = nx / 8, by = ny / 8, bz = nz / 8;
  const uint64_t nb = (uint64_t)bx * by * bz;
  const int lane = threadIdx.x & 31;
  const uint64_t wstride = (uint64_t)gridDim.x * (blockDim.x >> 5);
  for (uint64_t b = blockIdx.x * (uint64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); b < nb; b += wstride) {
    const int X = (int)(b % bx), Y = (int)((b / bx) % by), Z = (int)(b / ((uint64_t)bx * by));
    bool any = false;
    for (int k = 0; k < 16; k++) {
      const int i = lane + 32 * k;
      const size_t g = (size_t)(X * 8 + (i & 7)) + (size_t)nx * ((size_t)(Y * 8 + ((i >> 3) & 7)) + (size_t)ny * (Z * 8 + (i >> 6)));
      any |= grid[g] != 0;
    }
    const bool f = __any_sync(kFull, any);
    if (lane == 0) flags[b] = f ? 1 : 0;
  }
}

template <typename T>
__global__ void dense_fill_kernel(const T* grid, int nx, int ny, int nz, const uint32_t* ptr, uint64_t* occ,
                                  uint16_t* mat) {
  const int bx = nx / 8, by = ny / 8, bz = nz / 8;
  const uint64_t nb = (uint64_t)bx * by * bz;
  const int lane = threadIdx.x & 31;
  const uint64_t wstride = (uint64_t)gridDim.x * (blockDim.x >> 5);
  for (uint64_t b = blockIdx.x * (uint64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); b < nb; b += wstride) {
    const uint32_t slot = ptr[b];
    if (slot == MESO_EMPTY_BRICK) continue;
    const int X = (int)(b % bx), Y = (int)((b / bx) % by), Z = (int)(b / ((uint64_t)bx * by));
    for (int k = 0; k < 16; k++) {
      const int i = lane + 32 * k;
      const size_t g = (size_t)(X * 8 + (i & 7)) + (size_t)nx * ((size_t)(Y * 8 + ((i >> 3) & 7)) + (size_t)ny * (Z * 8 + (i >> 6)));
      const uint16_t m = (uint16_t)grid[g];
      mat[(size_t)slot * 512 + i] = m;
      const uint32_t bits = __ballot_sync(kFull, m != 0);
      if (lane == 0) reinterpret_cast<uint32_t*>(occ + (size_t)slot * 8)[k] = bits;
    }
  }
}

// ------------------------------------------------------------- generators
__global__ void dense_u8_kernel(int nx, int ny, int nz, uint32_t seed, uint8_t* out) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= (uint64_t)nx * ny * nz) return;
  const uint32_t x = (uint32_t)(i % nx), y = (uint32_t)((i / nx) % ny), z = (uint32_t)(i / ((uint64_t)nx * ny));
  const float n0 = vnoise3(x, y, z, 64, seed);
  float n1 = vnoise3(x, y, z, 32, seed + 1);
  float n2 = vnoise3(x, y, z, 16, seed + 2);
  float s = n0;
  n1 = __fmul_rn(n1, 0.5f);
  s = __fadd_rn(s, n1);
  n2 = __fmul_rn(n2, 0.25f);
  s = __fadd_rn(s, n2);
  s = __fdiv_rn(s, 1.75f);
  uint8_t m = 0;
  if (s > 0.5f) m = (uint8_t)(1 + (int)floorf(__fmul_rn(s, 15.0f)));
  out[i] = m;
}

// One CTA (1024 threads) per standalone chunk: keys = 17-bit quantised value
// noise (period 8) over (32767 - index), the k-th largest key found by a
// 4-pass radix select, solid iff key >= it; material 1 + hash mod m.
__global__ void __launch_bounds__(1024) chunks_u16_kernel(uint32_t seed0, const uint32_t* targets, uint16_t* out,
                                                          uint32_t* solid_count) {
  extern __shared__ uint32_t keys[];  // 32768
  __shared__ uint32_t hist[256];
  __shared__ uint32_t s_prefix, s_k;
  const uint32_t c = blockIdx.x, seed = seed0 + c;
  const uint32_t k = targets[c];
  for (uint32_t i = threadIdx.x; i < 32768u; i += blockDim.x) {
    const float n = vnoise3(i & 31u, (i >> 5) & 31u, i >> 10, 8, seed);
    uint32_t q = (uint32_t)floorf(__fmul_rn(n, 131072.0f));
    if (q > 131071u) q = 131071u;
    keys[i] = (q << 15) | (32767u - i);
  }
  uint32_t prefix = 0, pmask = 0, kk = k;
  for (int shift = 24; shift >= 0 && k > 0; shift -= 8) {
    for (int i = threadIdx.x; i < 256; i += blockDim.x) hist[i] = 0;
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < 32768u; i += blockDim.x) {
      const uint32_t key = keys[i];
      if ((key & pmask) == prefix) atomicAdd(&hist[(key >> shift) & 255u], 1u);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      uint32_t cum = 0;
      for (int d = 255; d >= 0; d--) {
        if (cum + hist[d] >= kk) {
          prefix |= (uint32_t)d << shift;
          kk -= cum;
          break;
        }
        cum += hist[d];
      }
      s_prefix = prefix;
      s_k = kk;
    }
    __syncthreads();
    prefix = s_prefix;
    kk = s_k;
    pmask |= 255u << shift;
  }
  const uint32_t m = 1u + pcg3d(seed, 0x77u, 0x3u) % 64u;
  uint16_t* dst = out + (size_t)c * 32768u;
  for (uint32_t i = threadIdx.x; i < 32768u; i += blockDim.x) {
    const bool solid = k > 0 && keys[i] >= prefix;
    dst[i] = solid ? (uint16_t)(1u + pcg3d(i, seed, 0x9E37u) % m) : (uint16_t)0;
  }
  if (threadIdx.x == 0 && solid_count) solid_count[c] = k;
}

// ------------------------------------------------------------------ edits
struct EditParams {
  const meso_sphere_edit* spheres;
  uint32_t n_spheres;
  const uint32_t* bricks;  // touched linear brick indices
  uint32_t n_bricks;
  int32_t bx, by;
  uint32_t* ptr;
  uint64_t* occ;
  uint16_t* mat;
  uint16_t* temp;          // 512 per touched brick
  uint8_t* state;          // per touched brick: bit0 present, bit1 nonempty
  uint32_t* free_stack;
  int32_t* alloc;          // [0] bump, [1] top
  uint32_t capacity;
  uint32_t* err;
};

__global__ void edit_compute_kernel(EditParams P) {
  const int lane = threadIdx.x & 31;
  const uint32_t wi = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (wi >= P.n_bricks) return;
  const uint32_t b = P.bricks[wi];
  const int X = (int)(b % P.bx) * 8, Y = (int)((b / P.bx) % P.by) * 8, Z = (int)(b / ((uint32_t)P.bx * P.by)) * 8;
  const uint32_t slot = P.ptr[b];
  const bool present = slot != MESO_EMPTY_BRICK;
  uint16_t v[16];
  for (int k = 0; k < 16; k++) v[k] = present ? P.mat[(size_t)slot * 512 + lane + 32 * k] : (uint16_t)0;
  for (uint32_t s = 0; s < P.n_spheres; s++) {
    const meso_sphere_edit e = P.spheres[s];
    const int r = e.radius;
    if (e.center[0] + r < X || e.center[0] - r > X + 7 || e.center[1] + r < Y || e.center[1] - r > Y + 7 ||
        e.center[2] + r < Z || e.center[2] - r > Z + 7)
      continue;
    const int r2 = r * r;
    for (int k = 0; k < 16; k++) {
      const int i = lane + 32 * k;
      const int dx = X + (i & 7) - e.center[0], dy = Y + ((i >> 3) & 7) - e.center[1], dz = Z + (i >> 6) - e.center[2];
      if (dx * dx + dy * dy + dz * dz <= r2) v[k] = e.material;
    }
  }
  bool any = false;
  for (int k = 0; k < 16; k++) any |= v[k] != 0;
  const bool nonempty = __any_sync(kFull, any);
  if (present && nonempty) {
    for (int k = 0; k < 16; k++) {
      P.mat[(size_t)slot * 512 + lane + 32 * k] = v[k];
      const uint32_t bits = __ballot_sync(kFull, v[k] != 0);
      if (lane == 0) reinterpret_cast<uint32_t*>(P.occ + (size_t)slot * 8)[k] = bits;
    }
  } else if (present && !nonempty) {
    if (lane == 0) {
      P.ptr[b] = MESO_EMPTY_BRICK;
      const int t = atomicAdd(&P.alloc[1], 1);
      P.free_stack[t] = slot;
    }
  } else if (!present && nonempty) {
    for (int k = 0; k < 16; k++) P.temp[(size_t)wi * 512 + lane + 32 * k] = v[k];
  }
  if (lane == 0) P.state[wi] = (uint8_t)((present ? 1 : 0) | (nonempty ? 2 : 0));
}

__global__ void edit_alloc_kernel(EditParams P) {
  const int lane = threadIdx.x & 31;
  const uint32_t wi = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (wi >= P.n_bricks) return;
  if (P.state[wi] != 2) return;  // absent and now nonempty
  uint32_t slot = 0;
  int ok = 1;
  if (lane == 0) {
    const int t = atomicSub(&P.alloc[1], 1) - 1;
    if (t >= 0) {
      slot = P.free_stack[t];
    } else {
      const int nb = atomicAdd(&P.alloc[0], 1);
      if ((uint32_t)nb >= P.capacity) {
        ok = 0;
        atomicOr(P.err, ERR_POOL_FULL);
      } else {
        slot = (uint32_t)nb;
      }
    }
  }
  ok = __shfl_sync(kFull, ok, 0);
  slot = __shfl_sync(kFull, slot, 0);
  if (!ok) return;
  const uint32_t b = P.bricks[wi];
  for (int k = 0; k < 16; k++) {
    const uint16_t m = P.temp[(size_t)wi * 512 + lane + 32 * k];
    P.mat[(size_t)slot * 512 + lane + 32 * k] = m;
    const uint32_t bits = __ballot_sync(kFull, m != 0);
    if (lane == 0) reinterpret_cast<uint32_t*>(P.occ + (size_t)slot * 8)[k] = bits;
  }
  if (lane == 0) P.ptr[b] = slot;
}

__global__ void edit_fix_kernel(int32_t* alloc, uint32_t capacity) {
  if (alloc[1] < 0) alloc[1] = 0;
  if ((uint32_t)alloc[0] > capacity) alloc[0] = (int32_t)capacity;
}

// Solid voxels of the live bricks: popcount of each linked brick's 8
// occupancy words, summed per warp and added to *count.
__global__ void count_solid_kernel(const uint32_t* ptr, uint64_t nb, const uint64_t* occ,
                                   unsigned long long* count) {
  uint32_t acc = 0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t b = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; b < nb; b += stride) {
    const uint32_t p = ptr[b];
    if (p == MESO_EMPTY_BRICK) continue;
    const uint4* w = reinterpret_cast<const uint4*>(occ + (size_t)p * 8);
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const uint4 v = w[k];
      acc += __popc(v.x) + __popc(v.y) + __popc(v.z) + __popc(v.w);
    }
  }
  const uint32_t tot = __reduce_add_sync(kFull, acc);
  if ((threadIdx.x & 31) == 0 && tot) atomicAdd(count, (unsigned long long)tot);
}

unsigned grid_for(uint64_t warps, int threads = 256) {
  const uint64_t per = threads / 32;
  uint64_t b = (warps + per - 1) / per;
  if (b > 1048576) b = 1048576;
  return (unsigned)(b ? b : 1);
}

}  // namespace

// One warp per macro cell (4x4x4 bricks): any occupied brick -> 1.
__global__ void macro_kernel(const uint32_t* ptr, int bx, int by, uint8_t* macro, const uint32_t* cells,
                             uint64_t n) {
  const uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= n) return;
  const uint32_t m = cells ? cells[w] : (uint32_t)w;
  const int mx = bx >> 2, my = by >> 2;
  const int cx = (int)(m % (uint32_t)mx), cy = (int)((m / (uint32_t)mx) % (uint32_t)my), cz = (int)(m / ((uint32_t)mx * my));
  bool any = false;
  for (int k = lane; k < 64; k += 32) {
    const int x = cx * 4 + (k & 3), y = cy * 4 + ((k >> 2) & 3), z = cz * 4 + (k >> 4);
    any |= ptr[(uint64_t)x + (uint64_t)bx * ((uint64_t)y + (uint64_t)by * z)] != MESO_EMPTY_BRICK;
  }
  const bool occupied = __any_sync(0xFFFFFFFFu, any);
  if (lane == 0) macro[m] = occupied ? 1 : 0;
}

// One warp per 16x16x16-brick cell: any occupied 4x4x4-brick child -> 1 (its
// 64 children read two per lane, at once); a cell that extends past the grid
// is marked 1 too, so no jump leaves the grid.
__global__ void macro2_kernel(const uint8_t* macro, int bx, int by, int bz, uint8_t* macro2, const uint32_t* list,
                              uint32_t n) {
  const int m2x = (bx + 15) / 16, m2y = (by + 15) / 16, m2z = (bz + 15) / 16;
  const uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= (list ? n : (uint64_t)m2x * m2y * m2z)) return;
  const uint32_t i = list ? list[w] : (uint32_t)w;
  const int cx = (int)(i % (uint32_t)m2x), cy = (int)((i / (uint32_t)m2x) % (uint32_t)m2y), cz = (int)(i / ((uint32_t)m2x * m2y));
  const int mx = bx / 4, my = by / 4, mz = bz / 4;
  const bool edge = (cx + 1) * 4 > mx || (cy + 1) * 4 > my || (cz + 1) * 4 > mz;
  bool any = false;
  if (!edge)
    for (int k = lane; k < 64; k += 32) {
      const int x = cx * 4 + (k & 3), y = cy * 4 + ((k >> 2) & 3), z = cz * 4 + (k >> 4);
      any |= macro[(uint32_t)x + (uint32_t)mx * ((uint32_t)y + (uint32_t)my * (uint32_t)z)] != 0;
    }
  const bool set = edge || __any_sync(0xFFFFFFFFu, any);
  if (lane == 0) macro2[i] = set ? 1 : 0;
}

// One warp per 64x64x64-brick cell: any nonzero 16x16x16 child, or a cell
// extending past the grid -> 1.
__global__ void macro3_kernel(const uint8_t* macro2, int bx, int by, int bz, uint8_t* macro3, const uint32_t* list,
                              uint32_t n) {
  const int m3x = (bx + 63) / 64, m3y = (by + 63) / 64, m3z = (bz + 63) / 64;
  const uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= (list ? n : (uint64_t)m3x * m3y * m3z)) return;
  const uint32_t i = list ? list[w] : (uint32_t)w;
  const int cx = (int)(i % (uint32_t)m3x), cy = (int)((i / (uint32_t)m3x) % (uint32_t)m3y), cz = (int)(i / ((uint32_t)m3x * m3y));
  const int m2x = (bx + 15) / 16, m2y = (by + 15) / 16;
  const bool edge = (cx + 1) * 64 > bx || (cy + 1) * 64 > by || (cz + 1) * 64 > bz;
  bool any = false;
  if (!edge)
    for (int k = lane; k < 64; k += 32) {
      const int x = cx * 4 + (k & 3), y = cy * 4 + ((k >> 2) & 3), z = cz * 4 + (k >> 4);
      any |= macro2[(uint32_t)x + (uint32_t)m2x * ((uint32_t)y + (uint32_t)m2y * (uint32_t)z)] != 0;
    }
  const bool set = edge || __any_sync(0xFFFFFFFFu, any);
  if (lane == 0) macro3[i] = set ? 1 : 0;
}

// ---------------------------------------------------------------- scene API

meso_status scene_alloc(meso_ctx* ctx, int32_t nx, int32_t ny, int32_t nz, uint64_t capacity, meso_scene** out) {
  meso_scene* s = new meso_scene();
  s->nx = nx;
  s->ny = ny;
  s->nz = nz;
  s->bx = nx / 8;
  s->by = ny / 8;
  s->bz = nz / 8;
  s->capacity = capacity;
  const uint64_t nb = n_bricks_of(s);
  const uint64_t bytes = nb * 4 + nb / 64 + n_macro2_of(s) + n_macro3_of(s) + capacity * (64 + 1024 + 4) + 16;
  if (ctx->budget_bytes && ctx->scene_bytes.load() + bytes > ctx->budget_bytes) {
    delete s;
    return fail(MESO_ERR_OVER_BUDGET, "scene exceeds the HBM budget");
  }
  cudaError_t e = cudaMalloc(&s->d_ptr, nb * 4);
  if (e == cudaSuccess) e = cudaMalloc(&s->d_macro, std::max<uint64_t>(nb / 64, 1));
  if (e == cudaSuccess) e = cudaMemset(s->d_macro, 0, std::max<uint64_t>(nb / 64, 1));
  if (e == cudaSuccess) e = cudaMalloc(&s->d_macro2, std::max<uint64_t>(n_macro2_of(s), 1));
  if (e == cudaSuccess) e = cudaMemset(s->d_macro2, 1, std::max<uint64_t>(n_macro2_of(s), 1));
  if (e == cudaSuccess) e = cudaMalloc(&s->d_macro3, std::max<uint64_t>(n_macro3_of(s), 1));
  if (e == cudaSuccess) e = cudaMemset(s->d_macro3, 1, std::max<uint64_t>(n_macro3_of(s), 1));
  if (e == cudaSuccess) e = cudaMalloc(&s->d_occ, std::max<uint64_t>(capacity, 1) * 64);
  if (e == cudaSuccess) e = cudaMalloc(&s->d_mat, std::max<uint64_t>(capacity, 1) * 1024);
  if (e == cudaSuccess) e = cudaMalloc(&s->d_free, std::max<uint64_t>(capacity, 1) * 4);
  if (e == cudaSuccess) e = cudaMalloc(&s->d_alloc, 16);
  if (e != cudaSuccess) {
    scene_release(ctx, s);
    cudaGetLastError();
    return fail(e == cudaErrorMemoryAllocation ? MESO_ERR_OOM : MESO_ERR_CUDA,
                std::string("scene allocation failed: ") + cudaGetErrorString(e));
  }
  s->bytes = bytes;
  ctx->scene_bytes.fetch_add(bytes);
  *out = s;
  return MESO_OK;
}

void scene_release(meso_ctx* ctx, meso_scene* s) {
  if (!s) return;
  cudaFree(s->d_ptr);
  cudaFree(s->d_macro);
  cudaFree(s->d_macro2);
  cudaFree(s->d_macro3);
  cudaFree(s->d_occ);
  cudaFree(s->d_mat);
  cudaFree(s->d_free);
  cudaFree(s->d_alloc);
  if (s->bytes) ctx->scene_bytes.fetch_sub(s->bytes);
  delete s;
}

meso_status rebuild_macro(meso_ctx* ctx, meso_scene* s, const uint32_t* d_cells, uint32_t n, cudaStream_t st,
                          const uint32_t* d_cells2, uint32_t n2, const uint32_t* d_cells3, uint32_t n3) {
  const uint64_t cells = d_cells ? n : n_macro_of(s);
  if (cells == 0) return MESO_OK;
  macro_kernel<<<(unsigned)((cells * 32 + 255) / 256), 256, 0, st>>>(s->d_ptr, s->bx, s->by, s->d_macro, d_cells,
                                                                     cells);
  const uint64_t cells2 = d_cells2 ? n2 : n_macro2_of(s);
  if (cells2)
    macro2_kernel<<<(unsigned)((cells2 * 32 + 255) / 256), 256, 0, st>>>(s->d_macro, s->bx, s->by, s->bz,
                                                                          s->d_macro2, d_cells2, n2);
  const uint64_t cells3 = d_cells3 ? n3 : n_macro3_of(s);
  if (cells3)
    macro3_kernel<<<(unsigned)((cells3 * 32 + 255) / 256), 256, 0, st>>>(s->d_macro2, s->bx, s->by, s->bz,
                                                                          s->d_macro3, d_cells3, n3);
  ctx->launches.fetch_add(3);
  MESO_CUDA_TRY(cudaGetLastError());
  return MESO_OK;
}

static meso_status finish_pools(meso_ctx* ctx, meso_scene* s, uint64_t count, cudaStream_t st) {
  MESO_TRY(rebuild_macro(ctx, s, nullptr, 0, st));
  int32_t init[4] = {(int32_t)count, 0, 0, 0};
  MESO_CUDA_TRY(cudaMemcpyAsync(s->d_alloc, init, 16, cudaMemcpyHostToDevice, st));
  MESO_CUDA_TRY(cudaStreamSynchronize(st));
  s->live_bricks_host = count;
  (void)ctx;
  return MESO_OK;
}

// Moves the pointer grid of a just-numbered scene into a fresh scene object
// sized count + spare.
static meso_status alloc_sized(meso_ctx* ctx, int32_t nx, int32_t ny, int32_t nz, uint64_t count, uint64_t spare,
                               meso_scene** out) {
  const uint64_t cap = count + spare;
  if (cap >= 0xFFFFFFFFull) return fail(MESO_ERR_INVALID_ARG, "brick pool too large");
  return scene_alloc(ctx, nx, ny, nz, cap, out);
}

meso_status scene_create_terrain(meso_ctx* ctx, const meso_terrain* t, uint64_t spare, meso_scene** out) {
  if (!t || !out) return fail(MESO_ERR_INVALID_ARG, "terrain: null argument");
  if (t->nx <= 0 || t->ny <= 0 || t->nz <= 0 || t->nx % 32 || t->ny % 32 || t->nz % 32 || t->nx > 8192 ||
      t->ny > 8192 || t->nz > 8192)
    return fail(MESO_ERR_INVALID_ARG, "terrain: dims must be positive multiples of 32 (<= 8192)");
  if (t->height_period == 0 || t->cave_period == 0 || t->height_octaves < 1 || t->height_octaves > 16)
    return fail(MESO_ERR_INVALID_ARG, "terrain: bad noise parameters");
  cudaStream_t st = ctx->stream;
  const TerrainDev T = to_dev(*t);
  const uint64_t ncol = (uint64_t)t->nx * t->ny;
  const int bx = t->nx / 8, by = t->ny / 8, bz = t->nz / 8;
  const uint64_t nb = (uint64_t)bx * by * bz;
  float* d_h = nullptr;
  float* d_hmax = nullptr;
  uint8_t* d_flags = nullptr;
  uint32_t* d_ptr_tmp = nullptr;
  cudaError_t ae = cudaMallocAsync(&d_h, ncol * 4, st);
  if (ae == cudaSuccess) ae = cudaMallocAsync(&d_hmax, (uint64_t)bx * by * 4, st);
  if (ae == cudaSuccess) ae = cudaMallocAsync(&d_flags, nb, st);
  if (ae == cudaSuccess) ae = cudaMallocAsync(&d_ptr_tmp, nb * 4, st);
  if (ae != cudaSuccess) {
    cudaFreeAsync(d_h, st);  // cudaFreeAsync(nullptr) is a no-op
    cudaFreeAsync(d_hmax, st);
    cudaFreeAsync(d_flags, st);
    cudaStreamSynchronize(st);
    return cuda_fail(ae, "terrain build: scratch allocation");
  }
  heights_kernel<<<(unsigned)((ncol + 255) / 256), 256, 0, st>>>(T, d_h);
  column_max_kernel<<<(bx * by + 255) / 256, 256, 0, st>>>(T, d_h, d_hmax);
  terrain_brick_kernel<false><<<grid_for(nb), 256, 0, st>>>(T, d_h, d_hmax, d_flags, nullptr, nullptr, nullptr);
  ctx->launches.fetch_add(3);
  uint64_t count = 0;
  meso_status rc = number_bricks(ctx, d_flags, nb, d_ptr_tmp, st, &count);
  meso_scene* s = nullptr;
  if (rc == MESO_OK) rc = alloc_sized(ctx, t->nx, t->ny, t->nz, count, spare, &s);
  if (rc == MESO_OK) {
    cudaMemcpyAsync(s->d_ptr, d_ptr_tmp, nb * 4, cudaMemcpyDeviceToDevice, st);
    terrain_brick_kernel<true><<<grid_for(nb), 256, 0, st>>>(T, d_h, d_hmax, d_flags, s->d_ptr, s->d_occ, s->d_mat);
    ctx->launches.fetch_add(1);
    rc = finish_pools(ctx, s, count, st);
  }
  cudaFreeAsync(d_h, st);
  cudaFreeAsync(d_hmax, st);
  cudaFreeAsync(d_flags, st);
  cudaFreeAsync(d_ptr_tmp, st);
  cudaError_t e = cudaStreamSynchronize(st);
  if (rc == MESO_OK && e != cudaSuccess) rc = cuda_fail(e, "terrain build");
  if (rc != MESO_OK) {
    scene_release(ctx, s);
    return rc;
  }
  *out = s;
  return MESO_OK;
}

// Brick map of a dense grid already in device memory (T = uint8_t or
// uint16_t; a uint8 material m becomes the uint16 material m).
template <typename T>
static meso_status build_from_device_grid(meso_ctx* ctx, const T* d_grid, int32_t nx, int32_t ny, int32_t nz,
                                          uint64_t spare, cudaStream_t st, meso_scene** out) {
  const uint64_t nb = (uint64_t)nx * ny * nz / 512;
  uint8_t* d_flags = nullptr;
  uint32_t* d_ptr_tmp = nullptr;
  cudaError_t ae = cudaMallocAsync(&d_flags, nb, st);
  if (ae == cudaSuccess) ae = cudaMallocAsync(&d_ptr_tmp, nb * 4, st);
  if (ae != cudaSuccess) {
    cudaFreeAsync(d_flags, st);  // cudaFreeAsync(nullptr) is a no-op
    cudaFreeAsync(d_ptr_tmp, st);
    cudaStreamSynchronize(st);
    return cuda_fail(ae, "dense scene: scratch allocation");
  }
  dense_flag_kernel<T><<<grid_for(nb), 256, 0, st>>>(d_grid, nx, ny, nz, d_flags);
  ctx->launches.fetch_add(1);
  uint64_t count = 0;
  meso_status rc = number_bricks(ctx, d_flags, nb, d_ptr_tmp, st, &count);
  meso_scene* s = nullptr;
  if (rc == MESO_OK) rc = alloc_sized(ctx, nx, ny, nz, count, spare, &s);
  if (rc == MESO_OK) {
    cudaMemcpyAsync(s->d_ptr, d_ptr_tmp, nb * 4, cudaMemcpyDeviceToDevice, st);
    dense_fill_kernel<T><<<grid_for(nb), 256, 0, st>>>(d_grid, nx, ny, nz, s->d_ptr, s->d_occ, s->d_mat);
    ctx->launches.fetch_add(1);
    rc = finish_pools(ctx, s, count, st);
  }
  cudaFreeAsync(d_flags, st);
  cudaFreeAsync(d_ptr_tmp, st);
  cudaError_t e = cudaStreamSynchronize(st);
  if (rc == MESO_OK && e != cudaSuccess) rc = cuda_fail(e, "dense scene build");
  if (rc != MESO_OK) {
    scene_release(ctx, s);
    return rc;
  }
  *out = s;
  return MESO_OK;
}

static meso_status check_grid_dims(int32_t nx, int32_t ny, int32_t nz) {
  if (nx <= 0 || ny <= 0 || nz <= 0 || nx % 32 || ny % 32 || nz % 32 || nx > 8192 || ny > 8192 || nz > 8192)
    return fail(MESO_ERR_INVALID_ARG, "dense scene: dims must be positive multiples of 32 (<= 8192)");
  return MESO_OK;
}

meso_status scene_create_dense(meso_ctx* ctx, const uint16_t* h_grid, int32_t nx, int32_t ny, int32_t nz,
                               uint64_t spare, meso_scene** out) {
  if (!h_grid || !out) return fail(MESO_ERR_INVALID_ARG, "dense scene: null argument");
  MESO_TRY(check_grid_dims(nx, ny, nz));
  cudaStream_t st = ctx->stream;
  const uint64_t nvox = (uint64_t)nx * ny * nz;
  uint16_t* d_grid = nullptr;
  cudaError_t ae = cudaMallocAsync(&d_grid, nvox * 2, st);
  if (ae == cudaSuccess) ae = cudaMemcpyAsync(d_grid, h_grid, nvox * 2, cudaMemcpyHostToDevice, st);
  if (ae != cudaSuccess) {
    cudaFreeAsync(d_grid, st);
    cudaStreamSynchronize(st);
    return cuda_fail(ae, "dense scene: upload");
  }
  const meso_status rc = build_from_device_grid<uint16_t>(ctx, d_grid, nx, ny, nz, spare, st, out);
  cudaFreeAsync(d_grid, st);
  cudaStreamSynchronize(st);
  return rc;
}

meso_status scene_create_grid(meso_ctx* ctx, int32_t kind, const void* d_grid, int32_t nx, int32_t ny, int32_t nz,
                              uint64_t spare, meso_scene** out) {
  if (!d_grid || !out) return fail(MESO_ERR_INVALID_ARG, "grid scene: null argument");
  MESO_TRY(check_grid_dims(nx, ny, nz));
  if (kind == MESO_SRC_GRID_U8)
    return build_from_device_grid<uint8_t>(ctx, static_cast<const uint8_t*>(d_grid), nx, ny, nz, spare, ctx->stream,
                                           out);
  if (kind == MESO_SRC_GRID_U16)
    return build_from_device_grid<uint16_t>(ctx, static_cast<const uint16_t*>(d_grid), nx, ny, nz, spare,
                                            ctx->stream, out);
  return fail(MESO_ERR_INVALID_ARG, "grid scene: kind must be MESO_SRC_GRID_U8 or MESO_SRC_GRID_U16");
}

meso_status scene_count_solid(meso_ctx* ctx, const meso_scene* s, uint64_t* n_solid) {
  if (!s || !n_solid) return fail(MESO_ERR_INVALID_ARG, "scene_count_solid: null argument");
  cudaStream_t st = ctx->stream;
  unsigned long long* d = nullptr;
  MESO_CUDA_TRY(cudaMallocAsync(&d, 8, st));
  cudaError_t e = cudaMemsetAsync(d, 0, 8, st);
  const uint64_t nb = n_bricks_of(s);
  if (e == cudaSuccess) {
    count_solid_kernel<<<(unsigned)std::min<uint64_t>((nb + 255) / 256, (uint64_t)ctx->sm_count * 16), 256, 0, st>>>(
        s->d_ptr, nb, s->d_occ, d);
    ctx->launches.fetch_add(1);
    e = cudaGetLastError();
  }
  unsigned long long h = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d, 8, cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(d, st);
  const cudaError_t e2 = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = e2;
  if (e != cudaSuccess) return cuda_fail(e, "scene_count_solid");
  *n_solid = h;
  return MESO_OK;
}

meso_status generate_dense_u8(meso_ctx* ctx, int32_t nx, int32_t ny, int32_t nz, uint32_t seed, uint8_t* d_out,
                              cudaStream_t st) {
  if (!d_out || nx <= 0 || ny <= 0 || nz <= 0) return fail(MESO_ERR_INVALID_ARG, "generate_dense_u8: bad argument");
  const uint64_t n = (uint64_t)nx * ny * nz;
  dense_u8_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(nx, ny, nz, seed, d_out);
  ctx->launches.fetch_add(1);
  MESO_CUDA_TRY(cudaGetLastError());
  return MESO_OK;
}

uint32_t chunk_solid_target(uint32_t seed) {
  // round(32768 * p), p = exp(U(ln 0.001, ln 0.9)), U from the chunk seed
  auto pcg = [](uint32_t x, uint32_t y, uint32_t z) {
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
  };
  const double u = (double)(pcg(seed, 0xA5A5u, 0x1234u) >> 8) / 16777216.0;
  const double lo = std::log(0.001), hi = std::log(0.9);
  const double p = std::exp(lo + (hi - lo) * u);
  return (uint32_t)std::floor(32768.0 * p + 0.5);
}

meso_status generate_chunks_u16(meso_ctx* ctx, uint32_t n, uint32_t seed0, uint16_t* d_out, uint32_t* d_solid,
                                cudaStream_t st) {
  if (!d_out || n == 0) return fail(MESO_ERR_INVALID_ARG, "generate_chunks_u16: bad argument");
  std::vector<uint32_t> targets(n);
  for (uint32_t i = 0; i < n; i++) targets[i] = chunk_solid_target(seed0 + i);
  uint32_t* d_t = nullptr;
  MESO_CUDA_TRY(cudaMallocAsync(&d_t, 4ull * n, st));
  MESO_CUDA_TRY(cudaMemcpyAsync(d_t, targets.data(), 4ull * n, cudaMemcpyHostToDevice, st));
  static bool attr = false;
  if (!attr) {
    MESO_CUDA_TRY(cudaFuncSetAttribute(chunks_u16_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 131072));
    attr = true;
  }
  chunks_u16_kernel<<<n, 1024, 131072, st>>>(seed0, d_t, d_out, d_solid);
  ctx->launches.fetch_add(1);
  MESO_CUDA_TRY(cudaFreeAsync(d_t, st));
  MESO_CUDA_TRY(cudaStreamSynchronize(st));
  MESO_CUDA_TRY(cudaGetLastError());
  return MESO_OK;
}

// Host side of an edit: touched bricks (sorted unique) and dirty chunks.
// Cells (bricks or chunks, edge `shift` bits of voxels) that the boxes
// [lo, hi] of the spheres touch, as sorted unique linear indices of a grid
// of G cells.  Small sets are collected and sorted; when the boxes cover a
// sizeable part of the grid, a bitmap over the grid is marked and scanned
// instead, so the cost stays bounded by the grid size.
// The cells (2^shift voxels on a side, grid G) that the boxes [lo, hi]
// overlap, unique; sorted unless `any_order` (then sorted only when two boxes
// share a cell: boxes that share none enumerate disjoint cells, and the
// sort is the costly part for a few thousand cells).
static void touched_cells(const int64_t (*lo)[3], const int64_t (*hi)[3], uint32_t n, int shift, const int64_t G[3],
                          std::vector<uint32_t>& out, bool any_order = false) {
  out.clear();
  uint64_t volume = 0;
  for (uint32_t i = 0; i < n; i++) {
    if (lo[i][0] > hi[i][0] || lo[i][1] > hi[i][1] || lo[i][2] > hi[i][2]) continue;
    uint64_t v = 1;
    for (int a = 0; a < 3; a++) v *= (uint64_t)((hi[i][a] >> shift) - (lo[i][a] >> shift) + 1);
    volume += v;
  }
  const uint64_t total = (uint64_t)(G[0] * G[1] * G[2]);
  const bool bitmap = volume > total / 64;
  std::vector<uint64_t> bits;
  if (bitmap) bits.assign((size_t)((total + 63) / 64), 0);
  else out.reserve((size_t)volume);
  for (uint32_t i = 0; i < n; i++) {
    if (lo[i][0] > hi[i][0] || lo[i][1] > hi[i][1] || lo[i][2] > hi[i][2]) continue;
    for (int64_t z = lo[i][2] >> shift; z <= hi[i][2] >> shift; z++)
      for (int64_t y = lo[i][1] >> shift; y <= hi[i][1] >> shift; y++)
        for (int64_t x = lo[i][0] >> shift; x <= hi[i][0] >> shift; x++) {
          const uint64_t k = (uint64_t)(x + G[0] * (y + G[1] * z));
          if (bitmap) bits[k >> 6] |= 1ull << (k & 63);
          else out.push_back((uint32_t)k);
        }
  }
  if (bitmap) {
    for (size_t w = 0; w < bits.size(); w++)
      for (uint64_t m = bits[w]; m; m &= m - 1) out.push_back((uint32_t)(w * 64 + (uint64_t)__builtin_ctzll(m)));
  } else {
    bool shared = !any_order;
    for (uint32_t i = 0; i < n && !shared; i++) {
      if (lo[i][0] > hi[i][0] || lo[i][1] > hi[i][1] || lo[i][2] > hi[i][2]) continue;
      for (uint32_t j = i + 1; j < n && !shared; j++) {
        if (lo[j][0] > hi[j][0] || lo[j][1] > hi[j][1] || lo[j][2] > hi[j][2]) continue;
        bool all = true;
        for (int a = 0; a < 3; a++)
          all = all && std::max(lo[i][a] >> shift, lo[j][a] >> shift) <= std::min(hi[i][a] >> shift, hi[j][a] >> shift);
        shared = all;
      }
    }
    if (shared) {
      std::sort(out.begin(), out.end());
      out.erase(std::unique(out.begin(), out.end()), out.end());
    }
  }
}

// The bricks a set of sphere edits may change (the voxel boxes of the
// spheres) and the chunks to remesh (the boxes grown by one voxel, whose
// faces may change), both sorted by linear index.
// The bricks and chunks the spheres' boxes touch, and the cells of 4^3, 16^3
// and 64^3 bricks holding those bricks (all unique; all but the bricks sorted).  A cell holds a
// touched brick iff the box overlaps it, so the cells come from the boxes
// directly, at the cells' own granularity.
static void edit_sets(const meso_scene* s, const meso_sphere_edit* sp, uint32_t n, std::vector<uint32_t>& bricks,
                      std::vector<uint32_t>& chunks, std::vector<uint32_t> (&cells)[3]) {
  const int64_t N[3] = {s->nx, s->ny, s->nz};
  std::vector<int64_t> box((size_t)n * 12);
  auto lo = reinterpret_cast<int64_t (*)[3]>(box.data());
  auto hi = lo + n;
  auto clo = hi + n;
  auto chi = clo + n;
  for (uint32_t i = 0; i < n; i++)
    for (int a = 0; a < 3; a++) {
      lo[i][a] = std::max<int64_t>((int64_t)sp[i].center[a] - sp[i].radius, 0);
      hi[i][a] = std::min<int64_t>((int64_t)sp[i].center[a] + sp[i].radius, N[a] - 1);
      clo[i][a] = std::max<int64_t>((int64_t)sp[i].center[a] - sp[i].radius - 1, 0);
      chi[i][a] = std::min<int64_t>((int64_t)sp[i].center[a] + sp[i].radius + 1, N[a] - 1);
    }
  const int64_t B[3] = {s->bx, s->by, s->bz}, C[3] = {s->nx / 32, s->ny / 32, s->nz / 32};
  touched_cells(lo, hi, n, 3, B, bricks, /*any_order=*/true);  // the edit kernels take them in any order
  touched_cells(clo, chi, n, 5, C, chunks);
  for (int l = 0; l < 3; l++) {
    // cells of (4^(l+1))^3 bricks: 2^(5+2l) voxels on a side, grids as the cell maps index them
    const int64_t cell = 4ll << (2 * l);
    const int64_t G[3] = {l == 0 ? s->bx / 4 : (s->bx + cell - 1) / cell, l == 0 ? s->by / 4 : (s->by + cell - 1) / cell,
                          l == 0 ? s->bz / 4 : (s->bz + cell - 1) / cell};
    touched_cells(lo, hi, n, 5 + 2 * l, G, cells[l]);
  }
}

meso_status edit_spheres(meso_ctx* ctx, meso_scene* s, const meso_sphere_edit* h_sp, uint32_t n, uint32_t* h_dirty,
                         uint32_t dirty_cap, uint32_t* n_dirty, cudaStream_t st) {
  if (!s || (n && !h_sp)) return fail(MESO_ERR_INVALID_ARG, "edit: null argument");
  for (uint32_t i = 0; i < n; i++)
    if (h_sp[i].radius < 0 || h_sp[i].radius > 4096) return fail(MESO_ERR_INVALID_ARG, "edit: radius out of range");
  std::vector<uint32_t> bricks, chunks, cells[3];
  edit_sets(s, h_sp, n, bricks, chunks, cells);
  if (n_dirty) *n_dirty = (uint32_t)chunks.size();
  if (h_dirty) std::copy(chunks.begin(), chunks.begin() + std::min<size_t>(chunks.size(), dirty_cap), h_dirty);
  if (bricks.empty()) return chunks.size() > dirty_cap && h_dirty ? fail(MESO_ERR_OVERFLOW, "edit: dirty list overflow") : MESO_OK;
  const size_t nb = bricks.size();
  // only the emptiness bytes of the cells holding touched bricks are recomputed
  // device scratch: [spheres | bricks | cells | cells2 | cells3] uploaded in
  // one copy, then the per-brick temporaries
  const size_t nc = cells[0].size(), nc2 = cells[1].size(), nc3 = cells[2].size();
  const size_t up = n * sizeof(meso_sphere_edit) + 4 * (nb + nc + nc2 + nc3);
  const size_t up16 = (up + 15) & ~size_t(15);
  std::vector<uint8_t> h(up);
  std::memcpy(h.data(), h_sp, n * sizeof(meso_sphere_edit));
  size_t o = n * sizeof(meso_sphere_edit);
  std::memcpy(h.data() + o, bricks.data(), nb * 4);
  o += nb * 4;
  for (int l = 0; l < 3; l++) {
    std::memcpy(h.data() + o, cells[l].data(), cells[l].size() * 4);
    o += cells[l].size() * 4;
  }
  const size_t bytes = up16 + nb * 1024 + nb + 16;
  uint8_t* d = nullptr;
  MESO_CUDA_TRY(cudaMallocAsync(&d, bytes, st));
  meso_sphere_edit* d_sp = reinterpret_cast<meso_sphere_edit*>(d);
  uint32_t* d_b = reinterpret_cast<uint32_t*>(d + n * sizeof(meso_sphere_edit));
  uint32_t* d_cells = d_b + nb;
  uint32_t* d_cells2 = d_cells + nc;
  uint32_t* d_cells3 = d_cells2 + nc2;
  uint16_t* d_temp = reinterpret_cast<uint16_t*>(d + up16);
  uint8_t* d_state = reinterpret_cast<uint8_t*>(d_temp) + nb * 1024;
  const cudaError_t ce = cudaMemcpyAsync(d, h.data(), up, cudaMemcpyHostToDevice, st);
  if (ce != cudaSuccess) {
    cudaFreeAsync(d, st);
    return cuda_fail(ce, "edit: upload");
  }
  EditParams P;
  P.spheres = d_sp;
  P.n_spheres = n;
  P.bricks = d_b;
  P.n_bricks = (uint32_t)nb;
  P.bx = s->bx;
  P.by = s->by;
  P.ptr = s->d_ptr;
  P.occ = s->d_occ;
  P.mat = s->d_mat;
  P.temp = d_temp;
  P.state = d_state;
  P.free_stack = s->d_free;
  P.alloc = reinterpret_cast<int32_t*>(s->d_alloc);
  P.capacity = (uint32_t)s->capacity;
  P.err = ctx->d_scratch + 1;
  const unsigned blocks = (unsigned)((nb + 7) / 8);
  edit_compute_kernel<<<blocks, 256, 0, st>>>(P);
  edit_alloc_kernel<<<blocks, 256, 0, st>>>(P);
  edit_fix_kernel<<<1, 1, 0, st>>>(P.alloc, P.capacity);
  ctx->launches.fetch_add(3);
  const meso_status mrc =
      rebuild_macro(ctx, s, d_cells, (uint32_t)nc, st, d_cells2, (uint32_t)nc2, d_cells3, (uint32_t)nc3);
  MESO_CUDA_TRY(cudaFreeAsync(d, st));
  if (mrc != MESO_OK) return mrc;
  MESO_CUDA_TRY(cudaGetLastError());
  if (h_dirty && chunks.size() > dirty_cap) return fail(MESO_ERR_OVERFLOW, "edit: dirty list overflow");
  return MESO_OK;
}

}  // namespace meso
