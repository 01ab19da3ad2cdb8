/*
 * meso_oracle.c -- CPU oracle for greedy chunk meshing and two-level
 * brick-map raymarching.  TEST INFRASTRUCTURE ONLY (checker and timed CPU
 * baseline); the product library never links it.  Parity status: unpinned by
 * the reference (it has neither algorithm); see meso_oracle.h for the
 * published methods restated here and the reference conventions kept.
 *
 * Build: gcc -O2 -std=c11 -ffp-contract=off -fno-fast-math -fPIC -shared -pthread
 */
#include "meso_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

/* ======================================================================== */
/* noise                                                                     */
/* ======================================================================== */

/* pcg3d (Jarzynski & Olano 2020), returning the third lane. */
uint32_t mo_pcg3d(uint32_t x, uint32_t y, uint32_t z) {
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

/* Lattice value in [0,1): top 24 bits of the hash, exact in FP32. */
float mo_lattice(uint32_t ix, uint32_t iy, uint32_t iz, uint32_t seed) {
  uint32_t h = mo_pcg3d(ix + seed * 0x9E3779B9u, iy ^ (seed * 0x85EBCA6Bu), iz + seed * 0xC2B2AE35u);
  return (float)(h >> 8) * (1.0f / 16777216.0f);
}

/* Quintic fade t^3 (t (6t - 15) + 10), fixed operation order. */
static float mo_fade(float t) {
  float a = t * 6.0f;
  a = a - 15.0f;
  a = t * a;
  a = a + 10.0f;
  float b = t * t;
  b = b * t;
  return b * a;
}

static float mo_lerp(float a, float b, float t) {
  float d = b - a;
  d = d * t;
  return a + d;
}

/* Sample position inside a lattice cell: ((p mod P) + 1/2) / P. */
static float mo_cell_frac(uint32_t p, uint32_t period) {
  float f = (float)(p % period);
  f = f + 0.5f;
  return f / (float)period;
}

float mo_vnoise3(uint32_t x, uint32_t y, uint32_t z, uint32_t period, uint32_t seed) {
  uint32_t ix = x / period, iy = y / period, iz = z / period;
  float sx = mo_fade(mo_cell_frac(x, period));
  float sy = mo_fade(mo_cell_frac(y, period));
  float sz = mo_fade(mo_cell_frac(z, period));
  float c000 = mo_lattice(ix, iy, iz, seed), c100 = mo_lattice(ix + 1, iy, iz, seed);
  float c010 = mo_lattice(ix, iy + 1, iz, seed), c110 = mo_lattice(ix + 1, iy + 1, iz, seed);
  float c001 = mo_lattice(ix, iy, iz + 1, seed), c101 = mo_lattice(ix + 1, iy, iz + 1, seed);
  float c011 = mo_lattice(ix, iy + 1, iz + 1, seed), c111 = mo_lattice(ix + 1, iy + 1, iz + 1, seed);
  float x00 = mo_lerp(c000, c100, sx), x10 = mo_lerp(c010, c110, sx);
  float x01 = mo_lerp(c001, c101, sx), x11 = mo_lerp(c011, c111, sx);
  float y0 = mo_lerp(x00, x10, sy), y1 = mo_lerp(x01, x11, sy);
  return mo_lerp(y0, y1, sz);
}

/* 2-D value noise: the 3-D lattice on the plane iz = 0x5BD1E995. */
static float mo_vnoise2(uint32_t x, uint32_t y, uint32_t period, uint32_t seed) {
  uint32_t ix = x / period, iy = y / period;
  const uint32_t iz = 0x5BD1E995u;
  float sx = mo_fade(mo_cell_frac(x, period));
  float sy = mo_fade(mo_cell_frac(y, period));
  float c00 = mo_lattice(ix, iy, iz, seed), c10 = mo_lattice(ix + 1, iy, iz, seed);
  float c01 = mo_lattice(ix, iy + 1, iz, seed), c11 = mo_lattice(ix + 1, iy + 1, iz, seed);
  float x0 = mo_lerp(c00, c10, sx), x1 = mo_lerp(c01, c11, sx);
  return mo_lerp(x0, x1, sy);
}

/* fBm: octave o has period P >> o, amplitude 2^-o and seed seed+o; the sum is
 * divided by the amplitude total (2 - 2^(1-octaves)). */
float mo_fbm2(uint32_t x, uint32_t y, uint32_t period, int octaves, uint32_t seed) {
  float sum = 0.0f, amp = 1.0f, norm = 0.0f;
  for (int o = 0; o < octaves; o++) {
    uint32_t p = period >> o;
    if (p == 0) p = 1;
    float n = mo_vnoise2(x, y, p, seed + (uint32_t)o);
    n = amp * n;
    sum = sum + n;
    norm = norm + amp;
    amp = amp * 0.5f;
  }
  return sum / norm;
}

/* ======================================================================== */
/* thread pool (one task = one index from an atomic counter)                 */
/* ======================================================================== */

int mo_hardware_threads(void) {
  long n = sysconf(_SC_NPROCESSORS_ONLN);
  return n > 0 ? (int)n : 1;
}

typedef void (*mo_task_fn)(void* ctx, uint64_t index);
typedef struct {
  mo_task_fn fn;
  void* ctx;
  uint64_t n;
  _Atomic uint64_t next;
} mo_pool_job;

static void* mo_pool_worker(void* arg) {
  mo_pool_job* job = (mo_pool_job*)arg;
  for (;;) {
    uint64_t i = atomic_fetch_add(&job->next, 1);
    if (i >= job->n) break;
    job->fn(job->ctx, i);
  }
  return NULL;
}

static void mo_parallel_for(uint64_t n, int nthreads, mo_task_fn fn, void* ctx) {
  if (nthreads <= 0) nthreads = mo_hardware_threads();
  if ((uint64_t)nthreads > n) nthreads = (int)(n ? n : 1);
  mo_pool_job job;
  job.fn = fn;
  job.ctx = ctx;
  job.n = n;
  atomic_init(&job.next, 0);
  if (nthreads <= 1) {
    mo_pool_worker(&job);
    return;
  }
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
  int started = 0;
  for (int i = 0; i < nthreads - 1; i++) {
    if (pthread_create(&th[i], NULL, mo_pool_worker, &job) == 0) started++;
    else break;
  }
  mo_pool_worker(&job);
  for (int i = 0; i < started; i++) pthread_join(th[i], NULL);
  free(th);
}

/* ======================================================================== */
/* scene generators                                                          */
/* ======================================================================== */

typedef struct {
  int nx, ny, nz;
  uint32_t seed;
  uint8_t* out;
} mo_dense_ctx;

static void mo_dense_row(void* c, uint64_t row) {
  mo_dense_ctx* ctx = (mo_dense_ctx*)c;
  uint32_t z = (uint32_t)(row / (uint64_t)ctx->ny), y = (uint32_t)(row % (uint64_t)ctx->ny);
  for (uint32_t x = 0; x < (uint32_t)ctx->nx; x++) {
    float n0 = mo_vnoise3(x, y, z, 64, ctx->seed);
    float n1 = mo_vnoise3(x, y, z, 32, ctx->seed + 1);
    float n2 = mo_vnoise3(x, y, z, 16, ctx->seed + 2);
    float s = n0;
    n1 = n1 * 0.5f;
    s = s + n1;
    n2 = n2 * 0.25f;
    s = s + n2;
    s = s / 1.75f;
    uint8_t m = 0;
    if (s > 0.5f) {
      float q = s * 15.0f;
      m = (uint8_t)(1 + (int)floorf(q));
    }
    ctx->out[(uint64_t)row * (uint64_t)ctx->nx + x] = m;
  }
}

void mo_gen_dense_u8(int nx, int ny, int nz, uint32_t seed, uint8_t* out) {
  mo_dense_ctx ctx = {nx, ny, nz, seed, out};
  mo_parallel_for((uint64_t)ny * (uint64_t)nz, 0, mo_dense_row, &ctx);
}

/* Solid-voxel target of a standalone chunk: round(32768 * p) with
 * p = exp(U(ln 0.001, ln 0.9)), U from the chunk seed. */
uint32_t mo_chunk_solid_target(uint32_t seed) {
  double u = (double)(mo_pcg3d(seed, 0xA5A5u, 0x1234u) >> 8) / 16777216.0;
  double lo = log(0.001), hi = log(0.9);
  double p = exp(lo + (hi - lo) * u);
  return (uint32_t)floor(32768.0 * p + 0.5);
}

uint32_t mo_chunk_material_count(uint32_t seed) { return 1u + mo_pcg3d(seed, 0x77u, 0x3u) % 64u; }

static int mo_cmp_u32_desc(const void* a, const void* b) {
  uint32_t x = *(const uint32_t*)a, y = *(const uint32_t*)b;
  return x < y ? 1 : (x > y ? -1 : 0);
}

/* Noise key of voxel idx of a chunk: 17-bit quantised value noise (period 8)
 * over 15 bits of (32767 - idx), unique per voxel: larger key = more solid,
 * ties on the noise broken towards the lower linear index. */
static uint32_t mo_chunk_key(uint32_t idx, uint32_t seed) {
  uint32_t x = idx & 31u, y = (idx >> 5) & 31u, z = idx >> 10;
  float n = mo_vnoise3(x, y, z, 8, seed);
  float q = n * 131072.0f;
  uint32_t qi = (uint32_t)floorf(q);
  if (qi > 131071u) qi = 131071u;
  return (qi << 15) | (32767u - idx);
}

typedef struct {
  uint32_t seed0;
  uint16_t* out;
  uint32_t* solid;
} mo_chunks_ctx;

static void mo_chunk_task(void* c, uint64_t i) {
  mo_chunks_ctx* ctx = (mo_chunks_ctx*)c;
  uint32_t seed = ctx->seed0 + (uint32_t)i;
  uint32_t k = mo_chunk_solid_target(seed);
  uint32_t m = mo_chunk_material_count(seed);
  uint32_t* keys = (uint32_t*)malloc(32768 * sizeof(uint32_t));
  uint32_t* sorted = (uint32_t*)malloc(32768 * sizeof(uint32_t));
  for (uint32_t v = 0; v < 32768; v++) keys[v] = sorted[v] = mo_chunk_key(v, seed);
  qsort(sorted, 32768, sizeof(uint32_t), mo_cmp_u32_desc);
  uint16_t* dst = ctx->out + (uint64_t)i * 32768u;
  for (uint32_t v = 0; v < 32768; v++) {
    int solid = k > 0 && keys[v] >= sorted[k - 1];
    dst[v] = solid ? (uint16_t)(1u + mo_pcg3d(v, seed, 0x9E37u) % m) : 0;
  }
  if (ctx->solid) ctx->solid[i] = k;
  free(keys);
  free(sorted);
}

void mo_gen_chunks_u16(int n_chunks, uint32_t seed0, uint16_t* out, uint32_t* solid_count) {
  mo_chunks_ctx ctx = {seed0, out, solid_count};
  mo_parallel_for((uint64_t)n_chunks, 0, mo_chunk_task, &ctx);
}

float mo_terrain_height(const mo_terrain* t, uint32_t x, uint32_t y) {
  float f = mo_fbm2(x, y, t->height_period, t->height_octaves, t->seed);
  f = t->height_amp * f;
  return t->height_base + f;
}

/* Solid iff z < h and the cave noise does not exceed the threshold; material
 * 1 + ((floor(h) - z) / 4 mod 64). */
uint16_t mo_terrain_voxel(const mo_terrain* t, float h, uint32_t x, uint32_t y, uint32_t z) {
  if (!((float)z < h)) return 0;
  float c = mo_vnoise3(x, y, z, t->cave_period, t->seed + 100u);
  if (c > t->cave_threshold) return 0;
  int32_t depth = (int32_t)floorf(h) - (int32_t)z;
  return (uint16_t)(1 + ((depth >> 2) & 63));
}

typedef struct {
  const mo_terrain* t;
  float* heights;   /* nx*ny */
  float* brick_hmax; /* per brick column */
  uint8_t* flags;   /* per brick */
  mo_brickmap* bm;
  int32_t bx, by, bz;
} mo_terrain_ctx;

static void mo_height_row(void* c, uint64_t y) {
  mo_terrain_ctx* ctx = (mo_terrain_ctx*)c;
  for (int32_t x = 0; x < ctx->t->nx; x++)
    ctx->heights[y * (uint64_t)ctx->t->nx + (uint64_t)x] = mo_terrain_height(ctx->t, (uint32_t)x, (uint32_t)y);
}

static int mo_terrain_brick(const mo_terrain_ctx* ctx, int64_t b, uint64_t* occ, uint16_t* mat) {
  int32_t bx = (int32_t)(b % ctx->bx), by = (int32_t)((b / ctx->bx) % ctx->by),
          bz = (int32_t)(b / ((int64_t)ctx->bx * ctx->by));
  float hmax = ctx->brick_hmax[(int64_t)by * ctx->bx + bx];
  if (!((float)(bz * 8) < hmax)) return 0;
  int any = 0;
  for (int lz = 0; lz < 8; lz++) {
    uint64_t w = 0;
    for (int ly = 0; ly < 8; ly++)
      for (int lx = 0; lx < 8; lx++) {
        uint32_t x = (uint32_t)(bx * 8 + lx), y = (uint32_t)(by * 8 + ly), z = (uint32_t)(bz * 8 + lz);
        float h = ctx->heights[(uint64_t)y * (uint64_t)ctx->t->nx + x];
        uint16_t m = mo_terrain_voxel(ctx->t, h, x, y, z);
        if (mat) mat[lx + 8 * ly + 64 * lz] = m;
        if (m) {
          w |= 1ull << (lx + 8 * ly);
          any = 1;
          if (!occ && !mat) return 1;
        }
      }
    if (occ) occ[lz] = w;
  }
  return any;
}

static void mo_terrain_flag(void* c, uint64_t b) {
  mo_terrain_ctx* ctx = (mo_terrain_ctx*)c;
  ctx->flags[b] = (uint8_t)mo_terrain_brick(ctx, (int64_t)b, NULL, NULL);
}

static void mo_terrain_fill(void* c, uint64_t b) {
  mo_terrain_ctx* ctx = (mo_terrain_ctx*)c;
  uint32_t p = ctx->bm->ptr[b];
  if (p == MO_EMPTY_BRICK) return;
  mo_terrain_brick(ctx, (int64_t)b, ctx->bm->occ + 8ull * p, ctx->bm->mat + 512ull * p);
}

int mo_build_terrain(const mo_terrain* t, int nthreads, mo_brickmap* out) {
  memset(out, 0, sizeof(*out));
  if (t->nx % 8 || t->ny % 8 || t->nz % 8 || t->nx <= 0 || t->ny <= 0 || t->nz <= 0) return -1;
  mo_terrain_ctx ctx;
  memset(&ctx, 0, sizeof(ctx));
  ctx.t = t;
  ctx.bx = t->nx / 8;
  ctx.by = t->ny / 8;
  ctx.bz = t->nz / 8;
  uint64_t nb = (uint64_t)ctx.bx * ctx.by * ctx.bz;
  ctx.heights = (float*)malloc(sizeof(float) * (size_t)t->nx * (size_t)t->ny);
  ctx.brick_hmax = (float*)malloc(sizeof(float) * (size_t)ctx.bx * (size_t)ctx.by);
  ctx.flags = (uint8_t*)malloc((size_t)nb);
  if (!ctx.heights || !ctx.brick_hmax || !ctx.flags) return -2;
  mo_parallel_for((uint64_t)t->ny, nthreads, mo_height_row, &ctx);
  for (int32_t by = 0; by < ctx.by; by++)
    for (int32_t bx = 0; bx < ctx.bx; bx++) {
      float m = -INFINITY;
      for (int ly = 0; ly < 8; ly++)
        for (int lx = 0; lx < 8; lx++) {
          float h = ctx.heights[(size_t)(by * 8 + ly) * (size_t)t->nx + (size_t)(bx * 8 + lx)];
          if (h > m) m = h;
        }
      ctx.brick_hmax[(size_t)by * (size_t)ctx.bx + (size_t)bx] = m;
    }
  mo_parallel_for(nb, nthreads, mo_terrain_flag, &ctx);
  out->nx = t->nx;
  out->ny = t->ny;
  out->nz = t->nz;
  out->ptr = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)nb);
  uint64_t count = 0;
  for (uint64_t b = 0; b < nb; b++) out->ptr[b] = ctx.flags[b] ? (uint32_t)count++ : MO_EMPTY_BRICK;
  out->n_bricks = out->cap_bricks = count;
  out->occ = (uint64_t*)calloc((size_t)(count ? count : 1) * 8, sizeof(uint64_t));
  out->mat = (uint16_t*)calloc((size_t)(count ? count : 1) * 512, sizeof(uint16_t));
  ctx.bm = out;
  mo_parallel_for(nb, nthreads, mo_terrain_fill, &ctx);
  free(ctx.heights);
  free(ctx.brick_hmax);
  free(ctx.flags);
  return 0;
}

int mo_build_from_dense_u16(int nx, int ny, int nz, const uint16_t* grid, mo_brickmap* out) {
  memset(out, 0, sizeof(*out));
  if (nx % 8 || ny % 8 || nz % 8) return -1;
  int64_t bx = nx / 8, by = ny / 8, bz = nz / 8, nb = bx * by * bz;
  out->nx = nx;
  out->ny = ny;
  out->nz = nz;
  out->ptr = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)nb);
  uint64_t count = 0;
  for (int64_t b = 0; b < nb; b++) {
    int64_t X = b % bx, Y = (b / bx) % by, Z = b / (bx * by);
    int any = 0;
    for (int lz = 0; lz < 8 && !any; lz++)
      for (int ly = 0; ly < 8 && !any; ly++)
        for (int lx = 0; lx < 8; lx++)
          if (grid[(X * 8 + lx) + (Y * 8 + ly) * (int64_t)nx + (Z * 8 + lz) * (int64_t)nx * ny]) {
            any = 1;
            break;
          }
    out->ptr[b] = any ? (uint32_t)count++ : MO_EMPTY_BRICK;
  }
  out->n_bricks = out->cap_bricks = count;
  out->occ = (uint64_t*)calloc((size_t)(count ? count : 1) * 8, sizeof(uint64_t));
  out->mat = (uint16_t*)calloc((size_t)(count ? count : 1) * 512, sizeof(uint16_t));
  for (int64_t b = 0; b < nb; b++) {
    uint32_t p = out->ptr[b];
    if (p == MO_EMPTY_BRICK) continue;
    int64_t X = b % bx, Y = (b / bx) % by, Z = b / (bx * by);
    for (int lz = 0; lz < 8; lz++)
      for (int ly = 0; ly < 8; ly++)
        for (int lx = 0; lx < 8; lx++) {
          uint16_t m = grid[(X * 8 + lx) + (Y * 8 + ly) * (int64_t)nx + (Z * 8 + lz) * (int64_t)nx * ny];
          out->mat[512ull * p + (uint64_t)(lx + 8 * ly + 64 * lz)] = m;
          if (m) out->occ[8ull * p + (uint64_t)lz] |= 1ull << (lx + 8 * ly);
        }
  }
  return 0;
}

void mo_brickmap_free(mo_brickmap* bm) {
  free(bm->ptr);
  free(bm->occ);
  free(bm->mat);
  memset(bm, 0, sizeof(*bm));
}

uint16_t mo_brickmap_get(const mo_brickmap* bm, int64_t x, int64_t y, int64_t z) {
  if (x < 0 || y < 0 || z < 0 || x >= bm->nx || y >= bm->ny || z >= bm->nz) return 0;
  int64_t bx = bm->nx / 8, by = bm->ny / 8;
  uint32_t p = bm->ptr[(x >> 3) + (y >> 3) * bx + (z >> 3) * bx * by];
  if (p == MO_EMPTY_BRICK) return 0;
  return bm->mat[512ull * p + (uint64_t)((x & 7) + 8 * (y & 7) + 64 * (z & 7))];
}

void mo_brickmap_to_dense(const mo_brickmap* bm, uint16_t* out) {
  for (int64_t z = 0; z < bm->nz; z++)
    for (int64_t y = 0; y < bm->ny; y++)
      for (int64_t x = 0; x < bm->nx; x++)
        out[x + y * bm->nx + z * (int64_t)bm->nx * bm->ny] = mo_brickmap_get(bm, x, y, z);
}

/* ======================================================================== */
/* greedy meshing                                                            */
/* ======================================================================== */

uint64_t mo_pack_quad(uint32_t chunk, int dir, int x, int y, int z, int w, int h, uint16_t mat) {
  return ((uint64_t)(chunk & 0xFFFFFu) << 44) | ((uint64_t)dir << 41) | ((uint64_t)z << 36) |
         ((uint64_t)y << 31) | ((uint64_t)x << 26) | ((uint64_t)(w - 1) << 21) | ((uint64_t)(h - 1) << 16) |
         (uint64_t)mat;
}

/* Material of chunk-local voxel (x,y,z), x,y,z in [-1, 32]; 0 outside the
 * source's domain (standalone chunks: anything outside the chunk). */
static uint16_t mo_src_get(const mo_source* s, const int32_t cc[3], int x, int y, int z) {
  switch (s->kind) {
    case MO_SRC_CHUNKS_U16:
    case MO_SRC_CHUNKS_U8: {
      if (x < 0 || y < 0 || z < 0 || x >= 32 || y >= 32 || z >= 32) return 0;
      uint64_t i = (uint64_t)cc[0] * 32768u + (uint64_t)(x + 32 * y + 1024 * z);
      return s->kind == MO_SRC_CHUNKS_U16 ? ((const uint16_t*)s->data)[i] : ((const uint8_t*)s->data)[i];
    }
    case MO_SRC_GRID_U8:
    case MO_SRC_GRID_U16: {
      int64_t gx = (int64_t)cc[0] * 32 + x, gy = (int64_t)cc[1] * 32 + y, gz = (int64_t)cc[2] * 32 + z;
      if (gx < 0 || gy < 0 || gz < 0 || gx >= s->nx || gy >= s->ny || gz >= s->nz) return 0;
      uint64_t i = (uint64_t)gx + (uint64_t)gy * (uint64_t)s->nx + (uint64_t)gz * (uint64_t)s->nx * (uint64_t)s->ny;
      return s->kind == MO_SRC_GRID_U16 ? ((const uint16_t*)s->data)[i] : ((const uint8_t*)s->data)[i];
    }
    case MO_SRC_BRICKMAP:
      return mo_brickmap_get(s->bm, (int64_t)cc[0] * 32 + x, (int64_t)cc[1] * 32 + y, (int64_t)cc[2] * 32 + z);
  }
  return 0;
}

/* Padded 34^3 material cube, index (x+1) + 34 (y+1) + 34^2 (z+1). */
static void mo_load_padded(const mo_source* s, const int32_t cc[3], uint16_t* cube) {
  for (int z = -1; z <= 32; z++)
    for (int y = -1; y <= 32; y++)
      for (int x = -1; x <= 32; x++) {
        int interior = x >= 0 && y >= 0 && z >= 0 && x < 32 && y < 32 && z < 32;
        int face_halo = (x < 0 || x > 31) + (y < 0 || y > 31) + (z < 0 || z > 31) == 1;
        cube[(x + 1) + 34 * (y + 1) + 1156 * (z + 1)] =
            (interior || face_halo) ? mo_src_get(s, cc, x, y, z) : 0;
      }
}

static const int MO_UAX[3] = {1, 0, 0}; /* u axis for faces on axis a */
static const int MO_VAX[3] = {2, 2, 1}; /* v axis */

/* Lysenko greedy meshing on one chunk: for each direction and slice, label
 * the 32x32 face mask by material, scan rows v then columns u; at the first
 * unconsumed face grow the width along u while the material matches, then
 * grow the height along v while the whole width run matches; consume and
 * emit. */
static uint64_t mo_greedy_cube(const uint16_t* cube, uint32_t chunk_id, uint64_t* out, uint64_t cap) {
  uint64_t n = 0;
  uint16_t mask[32][32];
  for (int dir = 0; dir < 6; dir++) {
    int a = dir >> 1, sgn = (dir & 1) ? -1 : 1;
    int ua = MO_UAX[a], va = MO_VAX[a];
    for (int s = 0; s < 32; s++) {
      for (int v = 0; v < 32; v++)
        for (int u = 0; u < 32; u++) {
          int p[3];
          p[a] = s;
          p[ua] = u;
          p[va] = v;
          uint16_t m = cube[(p[0] + 1) + 34 * (p[1] + 1) + 1156 * (p[2] + 1)];
          int q[3] = {p[0], p[1], p[2]};
          q[a] += sgn;
          uint16_t nb = cube[(q[0] + 1) + 34 * (q[1] + 1) + 1156 * (q[2] + 1)];
          mask[v][u] = (m != 0 && nb == 0) ? m : 0;
        }
      for (int v = 0; v < 32; v++)
        for (int u = 0; u < 32; u++) {
          uint16_t m = mask[v][u];
          if (!m) continue;
          int w = 1;
          while (u + w < 32 && mask[v][u + w] == m) w++;
          int h = 1;
          while (v + h < 32) {
            int ok = 1;
            for (int k = 0; k < w; k++)
              if (mask[v + h][u + k] != m) {
                ok = 0;
                break;
              }
            if (!ok) break;
            h++;
          }
          for (int j = 0; j < h; j++)
            for (int k = 0; k < w; k++) mask[v + j][u + k] = 0;
          int p[3];
          p[a] = s;
          p[ua] = u;
          p[va] = v;
          if (n < cap) out[n] = mo_pack_quad(chunk_id, dir, p[0], p[1], p[2], w, h, m);
          n++;
        }
    }
  }
  return n;
}

uint64_t mo_mesh_chunk(const mo_source* src, const int32_t chunk_coord[3], uint32_t chunk_id, uint64_t* out,
                       uint64_t cap) {
  uint16_t* cube = (uint16_t*)malloc(sizeof(uint16_t) * 34 * 34 * 34);
  mo_load_padded(src, chunk_coord, cube);
  uint64_t n = mo_greedy_cube(cube, chunk_id, out, cap);
  free(cube);
  return n;
}

uint64_t mo_count_faces(const mo_source* src, const int32_t cc[3]) {
  uint64_t n = 0;
  for (int z = 0; z < 32; z++)
    for (int y = 0; y < 32; y++)
      for (int x = 0; x < 32; x++) {
        if (!mo_src_get(src, cc, x, y, z)) continue;
        n += !mo_src_get(src, cc, x + 1, y, z);
        n += !mo_src_get(src, cc, x - 1, y, z);
        n += !mo_src_get(src, cc, x, y + 1, z);
        n += !mo_src_get(src, cc, x, y - 1, z);
        n += !mo_src_get(src, cc, x, y, z + 1);
        n += !mo_src_get(src, cc, x, y, z - 1);
      }
  return n;
}

typedef struct {
  const mo_source* src;
  const int32_t* coords;
  uint64_t** bufs;
  uint64_t* counts;
} mo_mesh_ctx;

static void mo_mesh_task(void* c, uint64_t i) {
  mo_mesh_ctx* ctx = (mo_mesh_ctx*)c;
  int32_t cc[3];
  if (ctx->src->kind == MO_SRC_CHUNKS_U16 || ctx->src->kind == MO_SRC_CHUNKS_U8) {
    cc[0] = ctx->coords ? ctx->coords[3 * i] : (int32_t)i;
    cc[1] = cc[2] = 0;
  } else {
    cc[0] = ctx->coords[3 * i];
    cc[1] = ctx->coords[3 * i + 1];
    cc[2] = ctx->coords[3 * i + 2];
  }
  uint16_t* cube = (uint16_t*)malloc(sizeof(uint16_t) * 34 * 34 * 34);
  mo_load_padded(ctx->src, cc, cube);
  uint64_t cap = 6ull * 32 * 32 * 32;
  uint64_t* buf = (uint64_t*)malloc(sizeof(uint64_t) * cap);
  ctx->counts[i] = mo_greedy_cube(cube, (uint32_t)i, buf, cap);
  ctx->bufs[i] = buf;
  free(cube);
}

static int mo_cmp_u64(const void* a, const void* b) {
  uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
  return x < y ? -1 : (x > y ? 1 : 0);
}

uint64_t mo_mesh_chunks_mt(const mo_source* src, const int32_t* chunk_coords, uint32_t n, int nthreads,
                           uint64_t* out, uint64_t cap) {
  mo_mesh_ctx ctx;
  ctx.src = src;
  ctx.coords = chunk_coords;
  ctx.bufs = (uint64_t**)calloc(n ? n : 1, sizeof(uint64_t*));
  ctx.counts = (uint64_t*)calloc(n ? n : 1, sizeof(uint64_t));
  mo_parallel_for(n, nthreads, mo_mesh_task, &ctx);
  uint64_t total = 0;
  for (uint32_t i = 0; i < n; i++) {
    /* quads of one chunk come out of the greedy scan already in (dir, slice,
     * v, u) order; sort each chunk's list into (dir, z, y, x) order */
    qsort(ctx.bufs[i], (size_t)ctx.counts[i], sizeof(uint64_t), mo_cmp_u64);
    for (uint64_t k = 0; k < ctx.counts[i]; k++) {
      if (total + k < cap) out[total + k] = ctx.bufs[i][k];
    }
    total += ctx.counts[i];
    free(ctx.bufs[i]);
  }
  free(ctx.bufs);
  free(ctx.counts);
  return total;
}

/* ======================================================================== */
/* two-level DDA                                                             */
/* ======================================================================== */

/* Pixel ray: s_x = ((2px+1)/W - 1) tan(fov/2) aspect, s_y = (1 - (2py+1)/H)
 * tan(fov/2); d = normalize((forward + s_x right) + s_y up). */
void mo_camera_ray(const mo_camera* cam, uint32_t px, uint32_t py, float dir[3]) {
  float aspect = (float)cam->width / (float)cam->height;
  float sx = (float)(2u * px + 1u) / (float)cam->width;
  sx = sx - 1.0f;
  sx = sx * cam->tan_half_fov_y;
  sx = sx * aspect;
  float sy = (float)(2u * py + 1u) / (float)cam->height;
  sy = 1.0f - sy;
  sy = sy * cam->tan_half_fov_y;
  float d[3];
  for (int a = 0; a < 3; a++) {
    float r = cam->right[a] * sx;
    float u = cam->up[a] * sy;
    float v = cam->forward[a] + r;
    d[a] = v + u;
  }
  float n2 = d[0] * d[0];
  float t1 = d[1] * d[1];
  float t2 = d[2] * d[2];
  n2 = n2 + t1;
  n2 = n2 + t2;
  float len = sqrtf(n2);
  for (int a = 0; a < 3; a++) dir[a] = d[a] / len;
}

typedef struct {
  int hit;
  int64_t v[3];
  float t;
  int axis; /* entry axis, -1 none */
  uint32_t coarse, fine;
} mo_trav;

static int mo_argmin3(const float tm[3]) {
  int a = 0;
  if (tm[1] < tm[a]) a = 1;
  if (tm[2] < tm[a]) a = 2;
  return a;
}

/* Traversal from voxel v (absolute, inside the grid) at time t0.  Coordinates
 * of the ray are relative to the frame origin `base` (absolute voxel).  A
 * brick whose pointer is empty is crossed in one coarse step; inside an
 * occupied brick every voxel advance is one fine step.  Boundary times are
 * recomputed from integer coordinates at every step: t = (b - o) * (1/d). */
static void mo_traverse(const mo_brickmap* bm, const int64_t base[3], const float o[3], const float d[3],
                        const int64_t v0[3], float t0, int axis0, mo_trav* r) {
  const int64_t N[3] = {bm->nx, bm->ny, bm->nz};
  const int64_t NB[3] = {bm->nx / 8, bm->ny / 8, bm->nz / 8};
  int s[3];
  float inv[3];
  for (int a = 0; a < 3; a++) {
    s[a] = d[a] > 0.0f ? 1 : (d[a] < 0.0f ? -1 : 0);
    inv[a] = s[a] ? 1.0f / d[a] : 0.0f;
  }
  int64_t v[3] = {v0[0], v0[1], v0[2]};
  int64_t B[3] = {v[0] >> 3, v[1] >> 3, v[2] >> 3};
  float t = t0;
  int ea = axis0;
  uint32_t cs = 0, fs = 0;
  const uint32_t cap = (uint32_t)(4 * (N[0] + N[1] + N[2]) + 64);
  r->hit = 0;
  for (;;) {
    if (cs + fs > cap) break;
    uint32_t p = bm->ptr[B[0] + B[1] * NB[0] + B[2] * NB[0] * NB[1]];
    if (p == MO_EMPTY_BRICK) {
      float tm[3];
      for (int a = 0; a < 3; a++) {
        if (!s[a]) {
          tm[a] = INFINITY;
          continue;
        }
        int64_t bnd = (B[a] + (s[a] > 0 ? 1 : 0)) * 8 - base[a];
        float q = (float)bnd - o[a];
        tm[a] = q * inv[a];
      }
      int a = mo_argmin3(tm);
      B[a] += s[a];
      cs++;
      if (B[a] < 0 || B[a] >= NB[a]) break;
      t = tm[a];
      ea = a;
      v[a] = s[a] > 0 ? B[a] * 8 : B[a] * 8 + 7;
      for (int b = 0; b < 3; b++) {
        if (b == a) continue;
        float pb = d[b] * t;
        pb = o[b] + pb;
        int64_t vb = (int64_t)floorf(pb) + base[b];
        if (vb < B[b] * 8) vb = B[b] * 8;
        if (vb > B[b] * 8 + 7) vb = B[b] * 8 + 7;
        v[b] = vb;
      }
      continue;
    }
    const uint64_t* occ = bm->occ + 8ull * p;
    int left = 0;
    for (;;) {
      int lx = (int)(v[0] & 7), ly = (int)(v[1] & 7), lz = (int)(v[2] & 7);
      if ((occ[lz] >> (lx + 8 * ly)) & 1ull) {
        r->hit = 1;
        break;
      }
      float tm[3];
      for (int a = 0; a < 3; a++) {
        if (!s[a]) {
          tm[a] = INFINITY;
          continue;
        }
        int64_t bnd = v[a] + (s[a] > 0 ? 1 : 0) - base[a];
        float q = (float)bnd - o[a];
        tm[a] = q * inv[a];
      }
      int a = mo_argmin3(tm);
      v[a] += s[a];
      fs++;
      t = tm[a];
      ea = a;
      if ((v[a] >> 3) != B[a]) {
        B[a] += s[a];
        if (B[a] < 0 || B[a] >= NB[a]) left = 1;
        break;
      }
      if (cs + fs > cap) {
        left = 1;
        break;
      }
    }
    if (r->hit || left) break;
  }
  r->v[0] = v[0];
  r->v[1] = v[1];
  r->v[2] = v[2];
  r->t = t;
  r->axis = ea;
  r->coarse = cs;
  r->fine = fs;
  (void)N;
}

static void mo_sign_inv(const float d[3], int s[3], float inv[3]) {
  for (int a = 0; a < 3; a++) {
    s[a] = d[a] > 0.0f ? 1 : (d[a] < 0.0f ? -1 : 0);
    inv[a] = s[a] ? 1.0f / d[a] : 0.0f;
  }
}

void mo_trace_ray(const mo_brickmap* bm, const int32_t cam_chunk[3], const float o[3], const float d[3],
                  const float light[3], int shadow, mo_hit* hit) {
  const int64_t N[3] = {bm->nx, bm->ny, bm->nz};
  int64_t base[3] = {(int64_t)cam_chunk[0] * 32, (int64_t)cam_chunk[1] * 32, (int64_t)cam_chunk[2] * 32};
  hit->voxel = UINT64_MAX;
  hit->t = INFINITY;
  hit->material = 0;
  hit->face = 6;
  hit->shadow = 255;
  hit->steps = 0;
  hit->shadow_steps = 0;
  int s[3];
  float inv[3];
  mo_sign_inv(d, s, inv);
  /* slab test against the grid box [-base, N - base) */
  float tnear = -INFINITY, tfar = INFINITY;
  int ea = -1;
  for (int a = 0; a < 3; a++) {
    float lo = (float)(-base[a]), hi = (float)(N[a] - base[a]);
    if (!s[a]) {
      if (o[a] < lo || o[a] >= hi) return;
      continue;
    }
    float q1 = lo - o[a], q2 = hi - o[a];
    float t1 = q1 * inv[a], t2 = q2 * inv[a];
    float tn = s[a] > 0 ? t1 : t2, tf = s[a] > 0 ? t2 : t1;
    if (tn > tnear) {
      tnear = tn;
      ea = a;
    }
    if (tf < tfar) tfar = tf;
  }
  if (!(tnear < tfar) || !(tfar > 0.0f)) return;
  int64_t v[3];
  float t0;
  if (tnear > 0.0f) {
    t0 = tnear;
    for (int b = 0; b < 3; b++) {
      if (b == ea) {
        v[b] = s[b] > 0 ? 0 : N[b] - 1;
        continue;
      }
      float pb = d[b] * t0;
      pb = o[b] + pb;
      int64_t vb = (int64_t)floorf(pb) + base[b];
      if (vb < 0) vb = 0;
      if (vb > N[b] - 1) vb = N[b] - 1;
      v[b] = vb;
    }
  } else {
    t0 = 0.0f;
    ea = -1;
    for (int b = 0; b < 3; b++) {
      int64_t vb = (int64_t)floorf(o[b]) + base[b];
      if (vb < 0) vb = 0;
      if (vb > N[b] - 1) vb = N[b] - 1;
      v[b] = vb;
    }
  }
  mo_trav r;
  mo_traverse(bm, base, o, d, v, t0, ea, &r);
  hit->steps = r.fine | (r.coarse << 16);
  if (!r.hit) return;
  hit->voxel = (uint64_t)r.v[0] + (uint64_t)r.v[1] * (uint64_t)N[0] + (uint64_t)r.v[2] * (uint64_t)N[0] * (uint64_t)N[1];
  hit->t = r.t;
  hit->material = mo_brickmap_get(bm, r.v[0], r.v[1], r.v[2]);
  if (r.axis < 0) {
    hit->face = 6;
    return;
  }
  hit->face = (uint8_t)(2 * r.axis + (s[r.axis] > 0 ? 1 : 0));
  if (!shadow) return;
  /* shadow ray from the centre of the empty voxel across the hit face */
  int64_t S[3] = {r.v[0], r.v[1], r.v[2]};
  S[r.axis] -= s[r.axis];
  if (S[r.axis] < 0 || S[r.axis] >= N[r.axis]) {
    hit->shadow = 0;
    return;
  }
  const float so[3] = {0.5f, 0.5f, 0.5f};
  mo_trav sr;
  mo_traverse(bm, S, so, light, S, 0.0f, -1, &sr);
  hit->shadow = (uint8_t)(sr.hit ? 1 : 0);
  hit->shadow_steps = sr.fine | (sr.coarse << 16);
}

typedef struct {
  const mo_brickmap* bm;
  const mo_camera* cams;
  const float* light;
  int shadow;
  mo_hit* hits;
  uint32_t row0;
  uint32_t rows_per_view;
} mo_ray_ctx;

static void mo_ray_row(void* c, uint64_t task) {
  mo_ray_ctx* ctx = (mo_ray_ctx*)c;
  uint32_t view = (uint32_t)(task / ctx->rows_per_view);
  uint32_t row = (uint32_t)(task % ctx->rows_per_view);
  const mo_camera* cam = &ctx->cams[view];
  uint32_t py = ctx->row0 + row;
  mo_hit* out = ctx->hits;
  uint64_t off = 0;
  for (uint32_t v = 0; v < view; v++) off += (uint64_t)ctx->cams[v].width * ctx->cams[v].height;
  for (uint32_t px = 0; px < cam->width; px++) {
    float d[3];
    mo_camera_ray(cam, px, py, d);
    mo_trace_ray(ctx->bm, cam->origin_chunk, cam->origin_frac, d, ctx->light, ctx->shadow,
                 &out[off + (uint64_t)row * cam->width + px]);
  }
}

void mo_raymarch_mt(const mo_brickmap* bm, const mo_camera* cams, uint32_t n_views, const float light[3],
                    int shadow, int nthreads, mo_hit* hits) {
  for (uint32_t v = 0; v < n_views; v++) {
    mo_ray_ctx ctx = {bm, &cams[v], light, shadow, hits, 0, cams[v].height};
    uint64_t off = 0;
    for (uint32_t k = 0; k < v; k++) off += (uint64_t)cams[k].width * cams[k].height;
    ctx.hits = hits + off;
    mo_parallel_for(cams[v].height, nthreads, mo_ray_row, &ctx);
  }
}

void mo_raymarch_rows_mt(const mo_brickmap* bm, const mo_camera* cam, uint32_t row0, uint32_t n_rows,
                         const float light[3], int shadow, int nthreads, mo_hit* hits) {
  mo_ray_ctx ctx = {bm, cam, light, shadow, hits, row0, n_rows};
  mo_parallel_for(n_rows, nthreads, mo_ray_row, &ctx);
}

/* ======================================================================== */
/* edits                                                                     */
/* ======================================================================== */

static int mo_grow(mo_brickmap* bm) {
  uint64_t nc = bm->cap_bricks ? bm->cap_bricks * 2 : 64;
  uint64_t* o = (uint64_t*)realloc(bm->occ, sizeof(uint64_t) * 8 * (size_t)nc);
  if (!o) return -1;
  bm->occ = o;
  uint16_t* m = (uint16_t*)realloc(bm->mat, sizeof(uint16_t) * 512 * (size_t)nc);
  if (!m) return -1;
  bm->mat = m;
  bm->cap_bricks = nc;
  return 0;
}

static int mo_set_voxel(mo_brickmap* bm, int64_t x, int64_t y, int64_t z, uint16_t mval) {
  int64_t bx = bm->nx / 8, by = bm->ny / 8;
  uint64_t bi = (uint64_t)((x >> 3) + (y >> 3) * bx + (z >> 3) * bx * by);
  uint32_t p = bm->ptr[bi];
  if (p == MO_EMPTY_BRICK) {
    if (!mval) return 0;
    if (bm->n_bricks >= bm->cap_bricks && mo_grow(bm)) return -1;
    p = (uint32_t)bm->n_bricks++;
    memset(bm->occ + 8ull * p, 0, 64);
    memset(bm->mat + 512ull * p, 0, 1024);
    bm->ptr[bi] = p;
  }
  int l = (int)((x & 7) + 8 * (y & 7)), lz = (int)(z & 7);
  bm->mat[512ull * p + (uint64_t)(l + 64 * lz)] = mval;
  if (mval) bm->occ[8ull * p + (uint64_t)lz] |= 1ull << l;
  else bm->occ[8ull * p + (uint64_t)lz] &= ~(1ull << l);
  return 0;
}

int mo_edit_spheres(mo_brickmap* bm, const mo_sphere* s, uint32_t n) {
  for (uint32_t i = 0; i < n; i++) {
    int64_t r = s[i].radius, cx = s[i].center[0], cy = s[i].center[1], cz = s[i].center[2];
    int64_t r2 = r * r;
    for (int64_t z = cz - r; z <= cz + r; z++) {
      if (z < 0 || z >= bm->nz) continue;
      for (int64_t y = cy - r; y <= cy + r; y++) {
        if (y < 0 || y >= bm->ny) continue;
        for (int64_t x = cx - r; x <= cx + r; x++) {
          if (x < 0 || x >= bm->nx) continue;
          int64_t dx = x - cx, dy = y - cy, dz = z - cz;
          if (dx * dx + dy * dy + dz * dz > r2) continue;
          if (mo_set_voxel(bm, x, y, z, s[i].material)) return -1;
        }
      }
    }
  }
  /* unlink bricks left empty */
  int64_t nb = (int64_t)(bm->nx / 8) * (bm->ny / 8) * (bm->nz / 8);
  for (int64_t b = 0; b < nb; b++) {
    uint32_t p = bm->ptr[b];
    if (p == MO_EMPTY_BRICK) continue;
    uint64_t any = 0;
    for (int k = 0; k < 8; k++) any |= bm->occ[8ull * p + (uint64_t)k];
    if (!any) bm->ptr[b] = MO_EMPTY_BRICK;
  }
  return 0;
}

static int mo_cmp_u32(const void* a, const void* b) {
  uint32_t x = *(const uint32_t*)a, y = *(const uint32_t*)b;
  return x < y ? -1 : (x > y ? 1 : 0);
}

uint32_t mo_dirty_chunks(const mo_brickmap* bm, const mo_sphere* s, uint32_t n, uint32_t* out, uint32_t cap) {
  int64_t CX = bm->nx / 32, CY = bm->ny / 32, CZ = bm->nz / 32;
  uint64_t total = (uint64_t)CX * CY * CZ;
  uint8_t* mark = (uint8_t*)calloc((size_t)total, 1);
  for (uint32_t i = 0; i < n; i++) {
    int64_t lo[3], hi[3];
    const int64_t N[3] = {bm->nx, bm->ny, bm->nz};
    int empty = 0;
    for (int a = 0; a < 3; a++) {
      lo[a] = (int64_t)s[i].center[a] - s[i].radius - 1;
      hi[a] = (int64_t)s[i].center[a] + s[i].radius + 1;
      if (lo[a] < 0) lo[a] = 0;
      if (hi[a] > N[a] - 1) hi[a] = N[a] - 1;
      if (lo[a] > hi[a]) empty = 1;
    }
    if (empty) continue;
    for (int64_t z = lo[2] >> 5; z <= hi[2] >> 5; z++)
      for (int64_t y = lo[1] >> 5; y <= hi[1] >> 5; y++)
        for (int64_t x = lo[0] >> 5; x <= hi[0] >> 5; x++) mark[x + y * CX + z * CX * CY] = 1;
  }
  uint32_t c = 0;
  for (uint64_t k = 0; k < total; k++)
    if (mark[k]) {
      if (c < cap) out[c] = (uint32_t)k;
      c++;
    }
  free(mark);
  if (c <= cap) qsort(out, c, sizeof(uint32_t), mo_cmp_u32);
  return c;
}

/* ======================================================================== */
/* erosion pyramid (the reference's per-block loop, restated)               */
/* ======================================================================== */

void mo_erode_mips(const uint8_t* occ, int R, int depth, uint8_t* out) {
  const size_t n = (size_t)R * R * R;
  for (size_t i = 0; i < n; i++) out[i] = occ[i] != 0;
  for (int d = 1; d < depth; d++) {
    const uint8_t* last = out + (size_t)(d - 1) * n;
    uint8_t* cur = out + (size_t)d * n;
    memset(cur, 0, n);
    for (int z = 0; z < R; z++)
      for (int y = 0; y < R; y++)
        for (int x = 0; x < R; x++) {
          if (!occ[(size_t)x + (size_t)R * (y + (size_t)R * z)]) continue; /* only the chunk's blocks */
          /* bIsOutOfBoundThickness(Location, R, 1) -> not eroded-solid */
          if (x < 1 || x >= R - 1 || y < 1 || y >= R - 1 || z < 1 || z >= R - 1) continue;
          int solid = 1;
          for (int dz = -1; dz <= 1 && solid; dz++)
            for (int dy = -1; dy <= 1 && solid; dy++)
              for (int dx = -1; dx <= 1; dx++) {
                if (!dx && !dy && !dz) continue;
                if (!last[(size_t)(x + dx) + (size_t)R * ((y + dy) + (size_t)R * (z + dz))]) {
                  solid = 0;
                  break;
                }
              }
          cur[(size_t)x + (size_t)R * (y + (size_t)R * z)] = (uint8_t)solid;
        }
  }
}
