// downstream.cu -- the steps either side of the two hot paths:
//   * brick-map files (save / load a resident scene);
//   * quad -> vertex expansion for raster consumers;
//   * the reference's 26-neighbour occupancy erosion pyramid on device.
#include <cstdio>
#include <cstring>
#include <vector>

#include "meso_internal.h"

namespace meso {

namespace {

using namespace ::meso::dev;

constexpr uint32_t kFull = 0xFFFFFFFFu;

// ------------------------------------------------------------ vertices
// Plane axes per face direction: X faces u=y v=z; Y faces u=x v=z; Z faces u=x v=y.
// A CTA of kQvThreads threads writes kQvPer x kQvThreads consecutive
// vertices (4 per quad); in step k thread t makes vertex
// base + k*kQvThreads + t, so every warp store covers 512 contiguous bytes,
// and a thread's kQvPer quad loads are issued before any of them is used.
constexpr int kQvThreads = 256, kQvPer = 8;

__device__ __forceinline__ float4 quad_vertex(uint64_t q, int k, const int32_t* origins, uint32_t n_chunks,
                                              uint32_t* err) {
  const uint32_t chunk = (uint32_t)(q >> 44);
  const int dir = (int)((q >> 41) & 7u);
  const int lz = (int)((q >> 36) & 31u), ly = (int)((q >> 31) & 31u), lx = (int)((q >> 26) & 31u);
  const int w = (int)((q >> 21) & 31u) + 1, h = (int)((q >> 16) & 31u) + 1;
  const uint32_t mat = (uint32_t)(q & 0xFFFFu);
  int ox = 0, oy = 0, oz = 0;
  if (chunk < n_chunks) {
    ox = __ldg(origins + 3 * chunk) * 32;
    oy = __ldg(origins + 3 * chunk + 1) * 32;
    oz = __ldg(origins + 3 * chunk + 2) * 32;
  } else if (k == 0) {
    atomicOr(err, ERR_BAD_INPUT);
  }
  const int a = dir >> 1;
  const int plus = (dir & 1) == 0;
  // voxel origin in (a, u, v) coordinates
  int pa, u0, v0;
  if (a == 0) { pa = lx; u0 = ly; v0 = lz; }
  else if (a == 1) { pa = ly; u0 = lx; v0 = lz; }
  else { pa = lz; u0 = lx; v0 = ly; }
  const int plane = pa + (plus ? 1 : 0);
  // u x v points along +a for X and Z faces and along -a for Y faces; keep
  // the corner order when that matches the face normal, reverse it otherwise
  const bool natural = (a == 1) ? !plus : plus;
  // corners (u0,v0), (u0+w,v0), (u0+w,v0+h), (u0,v0+h)
  const int c = natural ? k : (4 - k) & 3;
  const int cu = (c == 1 || c == 2) ? u0 + w : u0;
  const int cv = c >= 2 ? v0 + h : v0;
  int x, y, z;
  if (a == 0) { x = plane; y = cu; z = cv; }
  else if (a == 1) { y = plane; x = cu; z = cv; }
  else { z = plane; x = cu; y = cv; }
  float4 vtx;
  vtx.x = (float)(ox + x);
  vtx.y = (float)(oy + y);
  vtx.z = (float)(oz + z);
  vtx.w = __uint_as_float(mat | (uint32_t)dir << 16 | (uint32_t)k << 19);
  return vtx;
}

__global__ void __launch_bounds__(kQvThreads) quads_to_vertices_kernel(const uint64_t* __restrict__ quads, uint64_t n,
                                                                     const int32_t* __restrict__ origins,
                                                                     uint32_t n_chunks, meso_vertex* __restrict__ out,
                                                                     uint32_t* err) {
  const uint64_t base = (uint64_t)blockIdx.x * (kQvPer * kQvThreads) + threadIdx.x;
  uint64_t q[kQvPer];
#pragma unroll
  for (int k = 0; k < kQvPer; k++) {
    const uint64_t i = (base + (uint64_t)k * kQvThreads) >> 2;
    q[k] = i < n ? __ldg(quads + i) : 0ull;
  }
#pragma unroll
  for (int k = 0; k < kQvPer; k++) {
    const uint64_t vi = base + (uint64_t)k * kQvThreads;
    if ((vi >> 2) < n) __stcs(reinterpret_cast<float4*>(out) + vi, quad_vertex(q[k], (int)(vi & 3u), origins, n_chunks, err));
  }
}

// ------------------------------------------------------------ erosion
struct ErodeParams {
  int32_t kind;
  const uint8_t* data;
  int32_t nx, ny, nz;
  const uint32_t* bptr;
  const uint64_t* bocc;
  int32_t bx, by, bz;
  const int32_t* coords;
  uint32_t n;
  uint32_t depth;
  uint32_t* out;
  uint32_t* err;
};

// Occupancy of chunk-local voxel (x, y, z) of chunk c (x from the lane).
__device__ __forceinline__ bool chunk_voxel(const ErodeParams& p, uint32_t c, int cx, int cy, int cz, int x, int y,
                                            int z) {
  switch (p.kind) {
    case MESO_SRC_CHUNKS_U16: {
      const uint32_t idx = p.coords ? (uint32_t)p.coords[c] : c;
      return reinterpret_cast<const uint16_t*>(p.data)[(size_t)idx * 32768u + (z * 32 + y) * 32 + x] != 0;
    }
    case MESO_SRC_CHUNKS_U8: {
      const uint32_t idx = p.coords ? (uint32_t)p.coords[c] : c;
      return p.data[(size_t)idx * 32768u + (z * 32 + y) * 32 + x] != 0;
    }
    case MESO_SRC_GRID_U8:
    case MESO_SRC_GRID_U16: {
      const size_t g = (size_t)(cx * 32 + x) + (size_t)p.nx * ((size_t)(cy * 32 + y) + (size_t)p.ny * (cz * 32 + z));
      return p.kind == MESO_SRC_GRID_U8 ? p.data[g] != 0 : reinterpret_cast<const uint16_t*>(p.data)[g] != 0;
    }
    default: {
      const int gx = cx * 32 + x, gy = cy * 32 + y, gz = cz * 32 + z;
      const uint32_t b = p.bptr[(size_t)(gx >> 3) + (size_t)p.bx * ((size_t)(gy >> 3) + (size_t)p.by * (gz >> 3))];
      if (b == MESO_EMPTY_BRICK) return false;
      return (p.bocc[(size_t)b * 8 + (gz & 7)] >> ((gx & 7) + 8 * (gy & 7))) & 1ull;
    }
  }
}

// One CTA (256 threads) per chunk.  Mip d from mip d-1 on bit rows (z, y):
// (R << 1) & (R >> 1) covers the two x neighbours of the own row, and
// Q & (Q << 1) & (Q >> 1) the three x positions of each of the 8 other rows.
constexpr int kErodeThreads = 256;
constexpr int kErodeBatch = 8;  // 16-byte loads a thread has in flight at once
static_assert(4096 % (kErodeBatch * kErodeThreads) == 0, "a uint16 chunk is whole batches of loads");

__global__ void __launch_bounds__(kErodeThreads) erode_kernel(const ErodeParams p) {
  __shared__ uint32_t mip0[1024], cur[1024], nxt[1024];
  const uint32_t c = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int cx = 0, cy = 0, cz = 0;
  const bool grid = p.kind == MESO_SRC_GRID_U8 || p.kind == MESO_SRC_GRID_U16 || p.kind == MESO_SRC_BRICKMAP;
  bool ok = true;
  if (grid) {
    cx = p.coords[3 * c];
    cy = p.coords[3 * c + 1];
    cz = p.coords[3 * c + 2];
    const int lx = p.kind == MESO_SRC_BRICKMAP ? p.bx / 4 : p.nx / 32;
    const int ly = p.kind == MESO_SRC_BRICKMAP ? p.by / 4 : p.ny / 32;
    const int lz = p.kind == MESO_SRC_BRICKMAP ? p.bz / 4 : p.nz / 32;
    ok = cx >= 0 && cy >= 0 && cz >= 0 && cx < lx && cy < ly && cz < lz;
  } else if (p.coords) {
    ok = (uint32_t)p.coords[c] < (uint32_t)p.nx;
  }
  uint32_t* out = p.out + (size_t)c * p.depth * 1024;
  if (!ok) {
    if (threadIdx.x == 0) atomicOr(p.err, ERR_BAD_INPUT);
    for (uint32_t i = threadIdx.x; i < p.depth * 1024; i += blockDim.x) out[i] = 0;
    return;
  }
  if (p.kind == MESO_SRC_CHUNKS_U16 || p.kind == MESO_SRC_CHUNKS_U8) {
    // contiguous chunk: 16-byte streaming loads, kErodeBatch per thread in
    // flight at once, each giving the occupancy bits of 8 (uint16) or 16
    // (uint8) consecutive voxels of a row, written to the row word in shared
    // memory as a byte or a half word (bit x = voxel x)
    const uint32_t idx = p.coords ? (uint32_t)p.coords[c] : c;
    if (p.kind == MESO_SRC_CHUNKS_U16) {
      const uint4* src = reinterpret_cast<const uint4*>(p.data + (size_t)idx * 65536u);
      uint8_t* dst = reinterpret_cast<uint8_t*>(mip0);
#pragma unroll
      for (int i0 = 0; i0 < 4096; i0 += kErodeBatch * kErodeThreads) {
        uint4 v[kErodeBatch];
#pragma unroll
        for (int j = 0; j < kErodeBatch; j++) v[j] = __ldcs(src + i0 + j * kErodeThreads + threadIdx.x);
#pragma unroll
        for (int j = 0; j < kErodeBatch; j++) {
          const uint32_t w[4] = {v[j].x, v[j].y, v[j].z, v[j].w};
          uint32_t b = 0;
#pragma unroll
          for (int k = 0; k < 4; k++)
            b |= ((w[k] & 0xFFFFu) != 0 ? 1u : 0u) << (2 * k) | ((w[k] >> 16) != 0 ? 2u : 0u) << (2 * k);
          dst[i0 + j * kErodeThreads + threadIdx.x] = (uint8_t)b;
        }
      }
    } else {
      const uint4* src = reinterpret_cast<const uint4*>(p.data + (size_t)idx * 32768u);
      uint16_t* dst = reinterpret_cast<uint16_t*>(mip0);
#pragma unroll
      for (int i = threadIdx.x; i < 2048; i += kErodeThreads) {
        const uint4 v = __ldcs(src + i);
        const uint32_t w[4] = {v.x, v.y, v.z, v.w};
        uint32_t b = 0;
#pragma unroll
        for (int k = 0; k < 4; k++)
#pragma unroll
          for (int j = 0; j < 4; j++) b |= (((w[k] >> (8 * j)) & 0xFFu) != 0 ? 1u : 0u) << (4 * k + j);
        dst[i] = (uint16_t)b;
      }
    }
  } else {
    for (int row = warp; row < 1024; row += kErodeThreads / 32) {
      const int z = row >> 5, y = row & 31;
      const uint32_t w = __ballot_sync(kFull, chunk_voxel(p, c, cx, cy, cz, lane, y, z));
      if (lane == 0) mip0[row] = w;
    }
  }
  __syncthreads();
  for (int row = threadIdx.x; row < 1024; row += blockDim.x) {
    cur[row] = mip0[row];
    out[row] = mip0[row];
  }
  __syncthreads();
  for (uint32_t d = 1; d < p.depth; d++) {
    for (int row = threadIdx.x; row < 1024; row += blockDim.x) {
      const int z = row >> 5, y = row & 31;
      uint32_t acc = 0;
      if (y >= 1 && y <= 30 && z >= 1 && z <= 30) {
        const uint32_t R = cur[row];
        acc = (R << 1) & (R >> 1);
#pragma unroll
        for (int dz = -1; dz <= 1; dz++)
#pragma unroll
          for (int dy = -1; dy <= 1; dy++) {
            if (dz == 0 && dy == 0) continue;
            const uint32_t Q = cur[row + dz * 32 + dy];
            acc &= Q & (Q << 1) & (Q >> 1);
          }
        acc &= mip0[row] & 0x7FFFFFFEu;
      }
      nxt[row] = acc;
      out[(size_t)d * 1024 + row] = acc;
    }
    __syncthreads();
    for (int row = threadIdx.x; row < 1024; row += blockDim.x) cur[row] = nxt[row];
    __syncthreads();
  }
}

}  // namespace
}  // namespace meso

using namespace meso;

extern "C" {

meso_status meso_quads_to_vertices(meso_ctx* ctx, const uint64_t* d_quads, uint64_t n, const int32_t* d_origins,
                                   uint32_t n_chunks, meso_vertex* d_out, void* stream) {
  if (!ctx || (n && (!d_quads || !d_origins || !d_out)))
    return fail(MESO_ERR_INVALID_ARG, "quads_to_vertices: null argument");
  if (n == 0) return MESO_OK;
  if (reinterpret_cast<uintptr_t>(d_out) & 15u)
    return fail(MESO_ERR_INVALID_ARG, "quads_to_vertices: output must be 16-byte aligned");
  const cudaStream_t st = pick_stream(ctx, stream);
  const uint64_t per_block = (uint64_t)kQvPer * kQvThreads;
  const uint64_t blocks = (4 * n + per_block - 1) / per_block;
  if (blocks > 0x7FFFFFFFull) return fail(MESO_ERR_INVALID_ARG, "quads_to_vertices: too many quads");
  quads_to_vertices_kernel<<<(unsigned)blocks, kQvThreads, 0, st>>>(d_quads, n, d_origins, n_chunks, d_out,
                                                                    ctx->d_scratch + 1);
  ctx->launches.fetch_add(1);
  MESO_CUDA_TRY(cudaGetLastError());
  return MESO_OK;
}

meso_status meso_erode_mips(meso_ctx* ctx, const meso_mesh_source* src, const int32_t* d_coords, uint32_t n,
                            uint32_t depth, uint32_t* d_out, void* stream) {
  if (!ctx || !src || (n && !d_out)) return fail(MESO_ERR_INVALID_ARG, "erode_mips: null argument");
  if (depth < 1 || depth > 8) return fail(MESO_ERR_INVALID_ARG, "erode_mips: depth must be 1..8");
  if (n == 0) return MESO_OK;
  if (n > 0x7FFFFFFFu) return fail(MESO_ERR_INVALID_ARG, "erode_mips: too many chunks");
  ErodeParams p;
  memset(&p, 0, sizeof(p));
  p.kind = src->kind;
  p.coords = d_coords;
  p.n = n;
  p.depth = depth;
  p.out = d_out;
  p.err = ctx->d_scratch + 1;
  if (src->kind == MESO_SRC_BRICKMAP) {
    if (!src->scene || !d_coords) return fail(MESO_ERR_INVALID_ARG, "erode_mips: brick map needs scene + coords");
    p.bptr = src->scene->d_ptr;
    p.bocc = src->scene->d_occ;
    p.bx = src->scene->bx;
    p.by = src->scene->by;
    p.bz = src->scene->bz;
  } else if (src->kind >= MESO_SRC_GRID_U8 && src->kind <= MESO_SRC_CHUNKS_U8) {
    if (!src->d_data) return fail(MESO_ERR_INVALID_ARG, "erode_mips: null data");
    const bool grid = src->kind == MESO_SRC_GRID_U8 || src->kind == MESO_SRC_GRID_U16;
    if (grid && (!d_coords || src->nx % 32 || src->ny % 32 || src->nz % 32))
      return fail(MESO_ERR_INVALID_ARG, "erode_mips: grid needs coords and dims multiple of 32");
    if (!grid && d_coords && src->nx <= 0)
      return fail(MESO_ERR_INVALID_ARG, "erode_mips: an index list needs nx = chunks in the array");
    if (!grid && (reinterpret_cast<uintptr_t>(src->d_data) & 15u))
      return fail(MESO_ERR_INVALID_ARG, "erode_mips: chunk array must be 16-byte aligned");
    p.data = static_cast<const uint8_t*>(src->d_data);
    p.nx = src->nx;
    p.ny = src->ny;
    p.nz = src->nz;
  } else {
    return fail(MESO_ERR_INVALID_ARG, "erode_mips: unknown source kind");
  }
  erode_kernel<<<n, kErodeThreads, 0, pick_stream(ctx, stream)>>>(p);
  ctx->launches.fetch_add(1);
  MESO_CUDA_TRY(cudaGetLastError());
  return MESO_OK;
}

meso_status meso_scene_save(meso_ctx* ctx, const meso_scene* s, const char* path) {
  if (!ctx || !s || !path) return fail(MESO_ERR_INVALID_ARG, "scene_save: null argument");
  const uint64_t nb = n_bricks_of(s);
  std::vector<uint32_t> ptr(nb);
  std::vector<uint64_t> occ(s->capacity * 8);
  std::vector<uint16_t> mat(s->capacity * 512);
  MESO_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  MESO_CUDA_TRY(cudaMemcpy(ptr.data(), s->d_ptr, nb * 4, cudaMemcpyDeviceToHost));
  MESO_CUDA_TRY(cudaMemcpy(occ.data(), s->d_occ, occ.size() * 8, cudaMemcpyDeviceToHost));
  MESO_CUDA_TRY(cudaMemcpy(mat.data(), s->d_mat, mat.size() * 2, cudaMemcpyDeviceToHost));
  FILE* f = fopen(path, "wb");
  if (!f) return fail(MESO_ERR_INVALID_ARG, std::string("scene_save: cannot open ") + path);
  uint64_t n = 0;
  for (uint64_t b = 0; b < nb; b++) n += ptr[b] != MESO_EMPTY_BRICK;
  char hdr[32];
  memset(hdr, 0, sizeof(hdr));
  memcpy(hdr, "MESOBRK1", 8);
  const uint32_t version = 1;
  memcpy(hdr + 8, &version, 4);
  memcpy(hdr + 12, &s->nx, 4);
  memcpy(hdr + 16, &s->ny, 4);
  memcpy(hdr + 20, &s->nz, 4);
  memcpy(hdr + 24, &n, 8);
  bool ok = fwrite(hdr, 1, 32, f) == 32;
  std::vector<uint32_t> order;
  order.reserve(n);
  std::vector<uint32_t> canon(nb);
  for (uint64_t b = 0; b < nb; b++) {
    if (ptr[b] == MESO_EMPTY_BRICK) {
      canon[b] = MESO_EMPTY_BRICK;
    } else {
      canon[b] = (uint32_t)order.size();
      order.push_back(ptr[b]);
    }
  }
  ok = ok && fwrite(canon.data(), 4, nb, f) == nb;
  for (uint64_t k = 0; ok && k < n; k++) ok = fwrite(&occ[(size_t)order[k] * 8], 8, 8, f) == 8;
  for (uint64_t k = 0; ok && k < n; k++) ok = fwrite(&mat[(size_t)order[k] * 512], 2, 512, f) == 512;
  ok = (fclose(f) == 0) && ok;
  return ok ? MESO_OK : fail(MESO_ERR_INVALID_ARG, std::string("scene_save: write failed: ") + path);
}

meso_status meso_scene_load(meso_ctx* ctx, const char* path, uint64_t spare, meso_scene** out) {
  if (!ctx || !path || !out) return fail(MESO_ERR_INVALID_ARG, "scene_load: null argument");
  FILE* f = fopen(path, "rb");
  if (!f) return fail(MESO_ERR_INVALID_ARG, std::string("scene_load: cannot open ") + path);
  char hdr[32];
  if (fread(hdr, 1, 32, f) != 32 || memcmp(hdr, "MESOBRK1", 8) != 0) {
    fclose(f);
    return fail(MESO_ERR_INVALID_ARG, "scene_load: not a brick-map file");
  }
  uint32_t version;
  int32_t nx, ny, nz;
  uint64_t n;
  memcpy(&version, hdr + 8, 4);
  memcpy(&nx, hdr + 12, 4);
  memcpy(&ny, hdr + 16, 4);
  memcpy(&nz, hdr + 20, 4);
  memcpy(&n, hdr + 24, 8);
  if (version != 1 || nx <= 0 || ny <= 0 || nz <= 0 || nx % 32 || ny % 32 || nz % 32 || nx > 8192 || ny > 8192 ||
      nz > 8192) {
    fclose(f);
    return fail(MESO_ERR_INVALID_ARG, "scene_load: unsupported header");
  }
  const uint64_t nb = (uint64_t)(nx / 8) * (ny / 8) * (nz / 8);
  if (n > nb) {
    fclose(f);
    return fail(MESO_ERR_INVALID_ARG, "scene_load: corrupt brick count");
  }
  std::vector<uint32_t> ptr(nb);
  std::vector<uint64_t> occ(n * 8);
  std::vector<uint16_t> mat(n * 512);
  bool ok = fread(ptr.data(), 4, nb, f) == nb && fread(occ.data(), 8, n * 8, f) == n * 8 &&
            fread(mat.data(), 2, n * 512, f) == n * 512;
  fclose(f);
  if (!ok) return fail(MESO_ERR_INVALID_ARG, "scene_load: truncated file");
  for (uint64_t b = 0; b < nb; b++)
    if (ptr[b] != MESO_EMPTY_BRICK && ptr[b] >= n) return fail(MESO_ERR_INVALID_ARG, "scene_load: bad brick pointer");
  meso_scene* s = nullptr;
  MESO_TRY(scene_alloc(ctx, nx, ny, nz, n + spare, &s));
  cudaError_t e = cudaMemcpy(s->d_ptr, ptr.data(), nb * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && n) e = cudaMemcpy(s->d_occ, occ.data(), n * 64, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && n) e = cudaMemcpy(s->d_mat, mat.data(), n * 1024, cudaMemcpyHostToDevice);
  const int32_t alloc[4] = {(int32_t)n, 0, 0, 0};
  if (e == cudaSuccess) e = cudaMemcpy(s->d_alloc, alloc, 16, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    scene_release(ctx, s);
    return cuda_fail(e, "scene_load: upload");
  }
  meso_status rc = rebuild_macro(ctx, s, nullptr, 0, ctx->stream);
  if (rc == MESO_OK) {
    e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "scene_load: macro map");
  }
  if (rc != MESO_OK) {
    scene_release(ctx, s);
    return rc;
  }
  s->live_bricks_host = n;
  *out = s;
  return MESO_OK;
}

}  // extern "C"
