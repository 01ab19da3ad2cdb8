// raymarch.cu -- two-level brick-map DDA with a fused shadow ray, sm_103a.
//
// Replaces the reference's render step: an instanced draw of MaxBlockCount
// 7-vertex imposter cubes whose vertex shader places each visible block
// relative to the chunk-rebased camera (Samples/SimpleVoxel.cpp:146-192, draw
// at :383-387).  Here every pixel is one thread; a warp covers a tw x (32/tw)
// pixel tile so neighbouring rays walk the same bricks; many views (cameras,
// scenes) share one launch through a per-view descriptor table.
//
// Traversal (Amanatides & Woo 1987, at two levels): bricks whose pointer is
// empty are crossed in one coarse step; inside an occupied brick every voxel
// advance is a fine step over the brick's 8x8x8 occupancy bits.  Boundary
// times are recomputed from integer coordinates at every step,
// t = (b - o) * (1/d), with correctly rounded single operations
// (__fsub_rn/__fmul_rn...) so the results are bit-identical to a host
// evaluation of the same sequence.  Equal boundary times break x < y < z.
#include <cstring>

#include "meso_internal.h"

namespace meso {

struct RayView {
  const uint32_t* ptr;
  const uint64_t* occ;
  const uint16_t* mat;
  const uint8_t* macro;   // per 4x4x4-brick cell: nonzero iff a brick of it is occupied
  const uint8_t* macro2;  // per 16x16x16-brick cell: nonzero iff a 4x4x4 cell of it is, or it leaves the grid
  const uint8_t* macro3;  // per 64x64x64-brick cell, likewise from the 16x16x16 cells
  int32_t nx, ny, nz;
  int32_t cam_chunk[3];
  float o[3];
  float fwd[3], right[3], up[3];
  float tan_half;
  float aspect;  // width / height, correctly rounded
  uint32_t width, height;
  uint32_t tiles_x;
  uint32_t tile_start;
  meso_hit* out;  // this view's width*height hit records, row major
};

namespace {

using namespace ::meso::dev;

constexpr int kInlineViews = 32;
constexpr int kPlain = 0, kStatsMode = 1, kHashMode = 2;
constexpr uint32_t kFullMask = 0xFFFFFFFFu;
constexpr float kInf = __builtin_huge_valf();

// splitmix64 finaliser (the hit checksum's mixing function)
__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  x ^= x >> 30;
  x *= 0xBF58476D1CE4E5B9ull;
  x ^= x >> 27;
  x *= 0x94D049BB133111EBull;
  x ^= x >> 31;
  return x;
}

struct InlineViews {
  RayView v[kInlineViews];
};

struct RayParams {
  const RayView* table;  // device table (n_views > kInlineViews) or null
  uint32_t n_views;
  uint32_t total_tiles;
  uint32_t tile_w, tile_h;
  float light[3];
  float inv_light[3];  // 1 / light per axis, correctly rounded (0 for a zero component)
  uint32_t shadow;
  uint64_t* stats;
  unsigned long long* hash;  // checksum instantiation: partial sums per view (see launch_raymarch)
  uint32_t order_mul;  // CTA b takes block (b * order_mul) mod gridDim.x (0: block b)
  uint32_t cta_rows;   // 1: the output is host memory; write whole CTA rows (see the kernel)
};

struct Trav {
  int hit;
  int vx, vy, vz;
  float t;
  int axis;
  uint32_t coarse, fine;
  uint32_t fetches, bricks;  // pointer fetches and occupied bricks entered (statistics only)
};

__device__ __forceinline__ float bound_time(int b, float o, float inv) {
  return __fmul_rn(__fsub_rn(__int2float_rn(b), o), inv);
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Brick steps the two-level DDA takes along a non-exit axis (sign s, brick
// B, next brick boundary nb) while it crosses an empty cell of (mask+1)^3
// bricks, up to the step that leaves the cell through another axis at time
// tE (c_first: this axis wins ties with the exit axis).  The DDA takes its
// boundary events in (time, axis x<y<z) order and one axis's events come at
// strictly increasing times, so these steps are the interior boundaries that
// precede the exit in that order: a prefix.  Its length is estimated from the
// position at tE and settled by exact boundary-time comparisons.
__device__ __forceinline__ int cell_steps(int s, int B, int mask, int nb, float o, float d, float inv, float tE,
                                          bool c_first) {
  if (s == 0) return 0;
  const int inner = s > 0 ? mask - (B & mask) : (B & mask);
  if (inner == 0) return 0;
  const float pos = __fmaf_rn(d, tE, o);  // an estimate only
  const float q = s > 0 ? __fsub_rn(pos, __int2float_rn(nb)) : __fsub_rn(__int2float_rn(nb), pos);
  int k = clampi((int)ceilf(__fmul_rn(q, 0.125f)), 0, inner);
  while (k > 0) {
    const float tj = bound_time(nb + 8 * s * (k - 1), o, inv);
    if (tj < tE || (tj == tE && c_first)) break;
    k--;
  }
  while (k < inner) {
    const float tj = bound_time(nb + 8 * s * k, o, inv);
    if (!(tj < tE || (tj == tE && c_first))) break;
    k++;
  }
  return k;
}

// Empty-cell level of brick B: 3 if its 64^3-brick cell is empty, 2 if its
// 16^3-brick cell is, 1 if its 4^3-brick cell is, else 0 (the three bytes
// are fetched together).
__device__ __forceinline__ int cell_level(const RayView& V, int Bx, int By, int Bz, int MX, int MY, int MX2, int MY2,
                                          int MX3, int MY3) {
  const uint8_t m3 = __ldg(V.macro3 + (Bx >> 6) + MX3 * ((By >> 6) + MY3 * (Bz >> 6)));
  const uint8_t m2 = __ldg(V.macro2 + (Bx >> 4) + MX2 * ((By >> 4) + MY2 * (Bz >> 4)));
  const uint8_t m1 = __ldg(V.macro + (Bx >> 2) + MX * ((By >> 2) + MY * (Bz >> 2)));
  return m3 == 0 ? 3 : (m2 == 0 ? 2 : (m1 == 0 ? 1 : 0));
}

// Walks from voxel (vx,vy,vz) (absolute, inside the grid) at time t, entered
// through axis ea (-1 none).  Ray coordinates are relative to the absolute
// voxel (bx0,by0,bz0); ix, iy, iz are 1/d per axis (0 where d is 0).
//
// The walk is the same sequence of float operations as a step-by-step
// recomputation, organised for issue efficiency: a boundary time is only
// recomputed for the axis that stepped (the others are unchanged values),
// the entry voxel of a brick is derived only when an occupied brick is
// reached, the pointer index is stepped incrementally, and the occupancy
// word of the current z layer stays in a register.
template <bool kStats>
__device__ __forceinline__ void traverse(const RayView& V, int bx0, int by0, int bz0, float ox, float oy, float oz,
                                         float dx, float dy, float dz, float ix, float iy, float iz, int vx, int vy,
                                         int vz, float t, int ea, Trav& r) {
  uint32_t n_fetch = 0, n_brick = 0;
  const int sx = dx > 0.0f ? 1 : (dx < 0.0f ? -1 : 0);
  const int sy = dy > 0.0f ? 1 : (dy < 0.0f ? -1 : 0);
  const int sz = dz > 0.0f ? 1 : (dz < 0.0f ? -1 : 0);
  const int px = sx > 0 ? 1 : 0, py = sy > 0 ? 1 : 0, pz = sz > 0 ? 1 : 0;
  const int NBx = V.nx >> 3, NBy = V.ny >> 3, NBz = V.nz >> 3;
  const int MX = NBx >> 2, MY = NBy >> 2;                  // cells of 4x4x4 bricks
  const int MX2 = (NBx + 15) >> 4, MY2 = (NBy + 15) >> 4;  // cells of 16x16x16 bricks
  const int MX3 = (NBx + 63) >> 6, MY3 = (NBy + 63) >> 6;  // cells of 64x64x64 bricks
  const uint32_t strideY = (uint32_t)NBx, strideZ = (uint32_t)NBx * (uint32_t)NBy;
  // signed index increments of one step along each axis
  const uint32_t dIx = (uint32_t)sx, dIy = (uint32_t)(sy * (int)strideY), dIz = (uint32_t)(sz * (int)strideZ);
  int Bx = vx >> 3, By = vy >> 3, Bz = vz >> 3;
  uint32_t idx = (uint32_t)Bx + strideY * (uint32_t)By + strideZ * (uint32_t)Bz;
  uint32_t cs = 0, fs = 0;
  const uint32_t cap = (uint32_t)(4 * (V.nx + V.ny + V.nz) + 64);
  r.hit = 0;
  for (;;) {
    if (cs + fs > cap) break;
    uint32_t p = __ldg(V.ptr + idx);
    if (kStats) {
      n_fetch++;
      n_brick += p != MESO_EMPTY_BRICK;
    }
    if (p == MESO_EMPTY_BRICK) {
      // ---- coarse: one step per empty brick; nb* = next brick boundary
      // (relative voxel coordinate) along each axis.  A cell of 4x4x4 empty
      // bricks is crossed in one jump (the timed kernel; the statistics
      // instantiation takes every brick step to count the fetches).
      int nbx = (Bx + px) * 8 - bx0, nby = (By + py) * 8 - by0, nbz = (Bz + pz) * 8 - bz0;
      float tx = sx ? bound_time(nbx, ox, ix) : kInf;
      float ty = sy ? bound_time(nby, oy, iy) : kInf;
      float tz = sz ? bound_time(nbz, oz, iz) : kInf;
      bool out = false;
      int a = ea;
      // cell level at the current brick: 3 / 2 / 1 = its 64^3- / 16^3- /
      // 4^3-brick cell is empty (the largest such), 0 = take brick steps
      int lvl = 0;
      if (!kStats) lvl = cell_level(V, Bx, By, Bz, MX, MY, MX2, MY2, MX3, MY3);
      bool stale = false;
      for (;;) {
        if (lvl) {
          const int sh = 2 * lvl, mask = (1 << sh) - 1;
          const float Tx = sx ? bound_time((((Bx >> sh) + px) << (sh + 3)) - bx0, ox, ix) : kInf;
          const float Ty = sy ? bound_time((((By >> sh) + py) << (sh + 3)) - by0, oy, iy) : kInf;
          const float Tz = sz ? bound_time((((Bz >> sh) + pz) << (sh + 3)) - bz0, oz, iz) : kInf;
          const bool my = Ty < Tx;
          float tE = my ? Ty : Tx;
          const bool mz = Tz < tE;
          tE = mz ? Tz : tE;
          const int aE = mz ? 2 : (my ? 1 : 0);
          // along the exit axis every brick up to the face, then the exit step
          const int Be = aE == 0 ? Bx : (aE == 1 ? By : Bz), se = aE == 0 ? sx : (aE == 1 ? sy : sz);
          const int ke = (se > 0 ? mask - (Be & mask) : (Be & mask)) + 1;
          const int kx = aE == 0 ? ke : cell_steps(sx, Bx, mask, nbx, ox, dx, ix, tE, true);
          const int ky = aE == 1 ? ke : cell_steps(sy, By, mask, nby, oy, dy, iy, tE, aE == 2);
          const int kz = aE == 2 ? ke : cell_steps(sz, Bz, mask, nbz, oz, dz, iz, tE, false);
          const uint32_t k = (uint32_t)(kx + ky + kz);
          if (cs + fs + k <= cap) {
            cs += k;
            t = tE;
            a = aE;
            Bx += sx * kx;
            By += sy * ky;
            Bz += sz * kz;
            idx += dIx * (uint32_t)kx + dIy * (uint32_t)ky + dIz * (uint32_t)kz;
            nbx += 8 * sx * kx;
            nby += 8 * sy * ky;
            nbz += 8 * sz * kz;
            stale = true;  // brick boundary times: recomputed if a brick step follows
            out = ((unsigned)Bx >= (unsigned)NBx) | ((unsigned)By >= (unsigned)NBy) | ((unsigned)Bz >= (unsigned)NBz);
            if (out || cs + fs > cap) break;
            p = __ldg(V.ptr + idx);
            lvl = cell_level(V, Bx, By, Bz, MX, MY, MX2, MY2, MX3, MY3);
            if (p != MESO_EMPTY_BRICK) break;
            continue;
          }
          lvl = 0;  // the jump would pass the step cap: take brick steps
        }
        if (stale) {
          tx = sx ? bound_time(nbx, ox, ix) : kInf;
          ty = sy ? bound_time(nby, oy, iy) : kInf;
          tz = sz ? bound_time(nbz, oz, iz) : kInf;
          stale = false;
        }
        const bool cy = ty < tx;
        float tm = cy ? ty : tx;
        const bool cz = tz < tm;
        tm = cz ? tz : tm;
        a = cz ? 2 : (cy ? 1 : 0);
        cs++;
        t = tm;
        const bool a0 = a == 0, a1 = a == 1, a2 = a == 2;
        Bx += a0 ? sx : 0;
        By += a1 ? sy : 0;
        Bz += a2 ? sz : 0;
        idx += a0 ? dIx : (a1 ? dIy : dIz);
        out = ((unsigned)Bx >= (unsigned)NBx) | ((unsigned)By >= (unsigned)NBy) | ((unsigned)Bz >= (unsigned)NBz);
        if (out || cs + fs > cap) break;
        p = __ldg(V.ptr + idx);
        if (kStats) {
          n_fetch++;
          n_brick += p != MESO_EMPTY_BRICK;
        } else {
          // entering a new cell: is it empty?
          const int cnew = a0 ? Bx : (a1 ? By : Bz);
          const int snew = a0 ? sx : (a1 ? sy : sz);
          if ((cnew & 3) == (snew > 0 ? 0 : 3)) lvl = cell_level(V, Bx, By, Bz, MX, MY, MX2, MY2, MX3, MY3);
        }
        // the next boundary time is computed while the pointer load is in
        // flight; an occupied brick recomputes its times from scratch
        nbx += a0 ? 8 * sx : 0;
        nby += a1 ? 8 * sy : 0;
        nbz += a2 ? 8 * sz : 0;
        const int nb = a0 ? nbx : (a1 ? nby : nbz);
        const float oo = a0 ? ox : (a1 ? oy : oz);
        const float ii = a0 ? ix : (a1 ? iy : iz);
        const float tn = bound_time(nb, oo, ii);
        tx = a0 ? tn : tx;
        ty = a1 ? tn : ty;
        tz = a2 ? tn : tz;
        if (p != MESO_EMPTY_BRICK) break;
      }
      ea = a;
      if (out || p == MESO_EMPTY_BRICK) break;
      // entry voxel of the occupied brick: exact along the stepped axis,
      // floor of the entry point (clamped into the brick) along the others
      const int fx = clampi((int)floorf(__fadd_rn(ox, __fmul_rn(dx, t))) + bx0, Bx * 8, Bx * 8 + 7);
      const int fy = clampi((int)floorf(__fadd_rn(oy, __fmul_rn(dy, t))) + by0, By * 8, By * 8 + 7);
      const int fz = clampi((int)floorf(__fadd_rn(oz, __fmul_rn(dz, t))) + bz0, Bz * 8, Bz * 8 + 7);
      vx = a == 0 ? (sx > 0 ? Bx * 8 : Bx * 8 + 7) : fx;
      vy = a == 1 ? (sy > 0 ? By * 8 : By * 8 + 7) : fy;
      vz = a == 2 ? (sz > 0 ? Bz * 8 : Bz * 8 + 7) : fz;
    }
    // ---- fine: voxel steps inside occupied brick p; nv* = next voxel
    // boundary (relative) along each axis
    if (cs + fs > cap) break;
    const uint64_t* occ = V.occ + (size_t)p * 8;
    uint64_t w = __ldg(occ + (vz & 7));
    int nvx = vx + px - bx0, nvy = vy + py - by0, nvz = vz + pz - bz0;
    float tx = sx ? bound_time(nvx, ox, ix) : kInf;
    float ty = sy ? bound_time(nvy, oy, iy) : kInf;
    float tz = sz ? bound_time(nvz, oz, iz) : kInf;
    bool left = false, exit_brick = false;
    for (;;) {
      if ((w >> ((vx & 7) + 8 * (vy & 7))) & 1ull) {
        r.hit = 1;
        break;
      }
      const bool cy = ty < tx;
      float tm = cy ? ty : tx;
      const bool cz = tz < tm;
      tm = cz ? tz : tm;
      const int a = cz ? 2 : (cy ? 1 : 0);
      fs++;
      t = tm;
      ea = a;
      const bool a0 = a == 0, a1 = a == 1, a2 = a == 2;
      vx += a0 ? sx : 0;
      vy += a1 ? sy : 0;
      vz += a2 ? sz : 0;
      // next z layer's word, in flight during the bookkeeping below (on a
      // brick exit it wraps within this brick's 8 words and is unused)
      if (a2) w = __ldg(occ + (vz & 7));
      const int c = a0 ? vx : (a1 ? vy : vz);
      const int cb = a0 ? Bx : (a1 ? By : Bz);
      exit_brick = (c >> 3) != cb;
      if (exit_brick) {
        Bx = vx >> 3;
        By = vy >> 3;
        Bz = vz >> 3;
        idx += a0 ? dIx : (a1 ? dIy : dIz);
        left = ((unsigned)Bx >= (unsigned)NBx) | ((unsigned)By >= (unsigned)NBy) | ((unsigned)Bz >= (unsigned)NBz);
        break;
      }
      nvx += a0 ? sx : 0;
      nvy += a1 ? sy : 0;
      nvz += a2 ? sz : 0;
      const int nv = a0 ? nvx : (a1 ? nvy : nvz);
      const float oo = a0 ? ox : (a1 ? oy : oz);
      const float ii = a0 ? ix : (a1 ? iy : iz);
      const float tn = bound_time(nv, oo, ii);
      tx = a0 ? tn : tx;
      ty = a1 ? tn : ty;
      tz = a2 ? tn : tz;
      if (cs + fs > cap) {
        left = true;
        break;
      }
    }
    if (r.hit || left) break;
  }
  r.vx = vx;
  r.vy = vy;
  r.vz = vz;
  r.t = t;
  r.axis = ea;
  r.coarse = cs;
  r.fine = fs;
  r.fetches = n_fetch;
  r.bricks = n_brick;
}

__device__ __forceinline__ void camera_ray(const RayView& V, uint32_t px, uint32_t py, float& dx, float& dy,
                                           float& dz) {
  const float fw = __uint2float_rn(V.width), fh = __uint2float_rn(V.height);
  const float aspect = V.aspect;
  float sxv = __fdiv_rn(__uint2float_rn(2u * px + 1u), fw);
  sxv = __fsub_rn(sxv, 1.0f);
  sxv = __fmul_rn(sxv, V.tan_half);
  sxv = __fmul_rn(sxv, aspect);
  float syv = __fdiv_rn(__uint2float_rn(2u * py + 1u), fh);
  syv = __fsub_rn(1.0f, syv);
  syv = __fmul_rn(syv, V.tan_half);
  float d0 = __fadd_rn(__fadd_rn(V.fwd[0], __fmul_rn(V.right[0], sxv)), __fmul_rn(V.up[0], syv));
  float d1 = __fadd_rn(__fadd_rn(V.fwd[1], __fmul_rn(V.right[1], sxv)), __fmul_rn(V.up[1], syv));
  float d2 = __fadd_rn(__fadd_rn(V.fwd[2], __fmul_rn(V.right[2], sxv)), __fmul_rn(V.up[2], syv));
  float n2 = __fmul_rn(d0, d0);
  n2 = __fadd_rn(n2, __fmul_rn(d1, d1));
  n2 = __fadd_rn(n2, __fmul_rn(d2, d2));
  const float len = __fsqrt_rn(n2);
  dx = __fdiv_rn(d0, len);
  dy = __fdiv_rn(d1, len);
  dz = __fdiv_rn(d2, len);
}

template <bool kStats>
__device__ __forceinline__ void trace_pixel(const RayView& V, uint32_t px, uint32_t py, const RayParams& P,
                                            meso_hit& h, uint32_t* st) {
  h.voxel = ~0ull;
  h.t = kInf;
  h.material = 0;
  h.face = 6;
  h.shadow = 255;
  h.steps = 0;
  h.shadow_steps = 0;
  float dx, dy, dz;
  camera_ray(V, px, py, dx, dy, dz);
  const int bx0 = V.cam_chunk[0] * 32, by0 = V.cam_chunk[1] * 32, bz0 = V.cam_chunk[2] * 32;
  const float ox = V.o[0], oy = V.o[1], oz = V.o[2];
  const int sx = dx > 0.0f ? 1 : (dx < 0.0f ? -1 : 0);
  const int sy = dy > 0.0f ? 1 : (dy < 0.0f ? -1 : 0);
  const int sz = dz > 0.0f ? 1 : (dz < 0.0f ? -1 : 0);
  const float ix = sx ? __fdiv_rn(1.0f, dx) : 0.0f;
  const float iy = sy ? __fdiv_rn(1.0f, dy) : 0.0f;
  const float iz = sz ? __fdiv_rn(1.0f, dz) : 0.0f;
  // slab test against [-base, N - base)
  float tnear = -kInf, tfar = kInf;
  int ea = -1;
  {
    const float lo = __int2float_rn(-bx0), hi = __int2float_rn(V.nx - bx0);
    if (!sx) {
      if (ox < lo || ox >= hi) return;
    } else {
      const float inv = ix;
      const float t1 = __fmul_rn(__fsub_rn(lo, ox), inv), t2 = __fmul_rn(__fsub_rn(hi, ox), inv);
      const float tn = sx > 0 ? t1 : t2, tf = sx > 0 ? t2 : t1;
      if (tn > tnear) { tnear = tn; ea = 0; }
      if (tf < tfar) tfar = tf;
    }
  }
  {
    const float lo = __int2float_rn(-by0), hi = __int2float_rn(V.ny - by0);
    if (!sy) {
      if (oy < lo || oy >= hi) return;
    } else {
      const float inv = iy;
      const float t1 = __fmul_rn(__fsub_rn(lo, oy), inv), t2 = __fmul_rn(__fsub_rn(hi, oy), inv);
      const float tn = sy > 0 ? t1 : t2, tf = sy > 0 ? t2 : t1;
      if (tn > tnear) { tnear = tn; ea = 1; }
      if (tf < tfar) tfar = tf;
    }
  }
  {
    const float lo = __int2float_rn(-bz0), hi = __int2float_rn(V.nz - bz0);
    if (!sz) {
      if (oz < lo || oz >= hi) return;
    } else {
      const float inv = iz;
      const float t1 = __fmul_rn(__fsub_rn(lo, oz), inv), t2 = __fmul_rn(__fsub_rn(hi, oz), inv);
      const float tn = sz > 0 ? t1 : t2, tf = sz > 0 ? t2 : t1;
      if (tn > tnear) { tnear = tn; ea = 2; }
      if (tf < tfar) tfar = tf;
    }
  }
  if (!(tnear < tfar) || !(tfar > 0.0f)) return;
  int vx, vy, vz;
  float t0;
  if (tnear > 0.0f) {
    t0 = tnear;
    vx = ea == 0 ? (sx > 0 ? 0 : V.nx - 1)
                 : clampi((int)floorf(__fadd_rn(ox, __fmul_rn(dx, t0))) + bx0, 0, V.nx - 1);
    vy = ea == 1 ? (sy > 0 ? 0 : V.ny - 1)
                 : clampi((int)floorf(__fadd_rn(oy, __fmul_rn(dy, t0))) + by0, 0, V.ny - 1);
    vz = ea == 2 ? (sz > 0 ? 0 : V.nz - 1)
                 : clampi((int)floorf(__fadd_rn(oz, __fmul_rn(dz, t0))) + bz0, 0, V.nz - 1);
  } else {
    t0 = 0.0f;
    ea = -1;
    vx = clampi((int)floorf(ox) + bx0, 0, V.nx - 1);
    vy = clampi((int)floorf(oy) + by0, 0, V.ny - 1);
    vz = clampi((int)floorf(oz) + bz0, 0, V.nz - 1);
  }
  Trav r;
  traverse<kStats>(V, bx0, by0, bz0, ox, oy, oz, dx, dy, dz, ix, iy, iz, vx, vy, vz, t0, ea, r);
  h.steps = r.fine | (r.coarse << 16);
  if (kStats) {
    st[0] += r.fetches;
    st[1] += r.bricks;
    st[3] += 1;
  }
  if (!r.hit) return;
  if (kStats) st[2] += 1;
  h.voxel = (uint64_t)r.vx + (uint64_t)V.nx * ((uint64_t)r.vy + (uint64_t)V.ny * (uint64_t)r.vz);
  h.t = r.t;
  {
    const uint32_t p =
        __ldg(V.ptr + (size_t)(r.vx >> 3) + (size_t)(V.nx >> 3) * ((size_t)(r.vy >> 3) + (size_t)(V.ny >> 3) * (r.vz >> 3)));
    h.material = __ldg(V.mat + (size_t)p * 512 + (r.vx & 7) + 8 * (r.vy & 7) + 64 * (r.vz & 7));
  }
  if (r.axis < 0) return;
  const int sa = r.axis == 0 ? sx : (r.axis == 1 ? sy : sz);
  h.face = (uint8_t)(2 * r.axis + (sa > 0 ? 1 : 0));
  if (!P.shadow) return;
  int Sx = r.vx, Sy = r.vy, Sz = r.vz;
  bool outside;
  if (r.axis == 0) { Sx -= sx; outside = Sx < 0 || Sx >= V.nx; }
  else if (r.axis == 1) { Sy -= sy; outside = Sy < 0 || Sy >= V.ny; }
  else { Sz -= sz; outside = Sz < 0 || Sz >= V.nz; }
  if (outside) {
    h.shadow = 0;
    return;
  }
  Trav sr;
  traverse<kStats>(V, Sx, Sy, Sz, 0.5f, 0.5f, 0.5f, P.light[0], P.light[1], P.light[2], P.inv_light[0],
                   P.inv_light[1], P.inv_light[2], Sx, Sy, Sz, 0.0f, -1, sr);
  if (kStats) {
    st[0] += sr.fetches;
    st[1] += sr.bricks;
    st[3] += 1;
  }
  h.shadow = (uint8_t)(sr.hit ? 1 : 0);
  h.shadow_steps = sr.fine | (sr.coarse << 16);
}


// kMode: kPlain; kStatsMode also accumulates {pointer fetches, occupied
// bricks entered, hits, rays} into P.stats; kHashMode also adds each view's
// order-sensitive hit checksum and its traced shadow rays into P.hash (the
// serving loop's per-request summary, so the hits need not be read again).
// Each is a separate instantiation; the timed path has none of it.
// At most 128 threads per CTA; 8 resident CTAs per SM cap registers at 64,
// which measured faster than the uncapped 73 (more warps to hide latency).
template <bool kInline, int kMode>
__global__ void __launch_bounds__(128, 8) raymarch_kernel(const RayParams P, const __grid_constant__ InlineViews iv) {
  constexpr bool kStats = kMode == kStatsMode;
  const uint32_t warps = blockDim.x >> 5;
  const uint32_t bid = P.order_mul ? (uint32_t)(((uint64_t)blockIdx.x * P.order_mul) % gridDim.x) : blockIdx.x;
  const uint32_t tile = bid * warps + (threadIdx.x >> 5);
  if (tile >= P.total_tiles) return;
  const int lane = threadIdx.x & 31;
  const RayView* views = kInline ? iv.v : P.table;
  // view lookup: last view whose tile_start <= tile
  uint32_t lo = 0, hi = P.n_views;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (views[mid].tile_start <= tile) lo = mid;
    else hi = mid;
  }
  const RayView& V = views[lo];
  const uint32_t lt = tile - V.tile_start;
  const uint32_t tx = lt % V.tiles_x, ty = lt / V.tiles_x;
  const uint32_t px0 = tx * P.tile_w, py0 = ty * P.tile_h;
  const uint32_t px = px0 + (uint32_t)lane % P.tile_w;
  const uint32_t py = py0 + (uint32_t)lane / P.tile_w;
  uint32_t st[4] = {0, 0, 0, 0};
  // The tile's hit records (24 B each) are staged in shared memory and
  // written back as runs of consecutive 8-byte words, one run per tile row,
  // so every store instruction fills whole sectors (this matters most when
  // the output is page-locked host memory written over the CPU-GPU link).
  __shared__ __align__(16) uint64_t stage[4][96];
  uint64_t* sw = stage[threadIdx.x >> 5];
  if (px < V.width && py < V.height) {
    meso_hit h;
    trace_pixel<kStats>(V, px, py, P, h, st);
    sw[3 * lane] = h.voxel;
    sw[3 * lane + 1] = (uint64_t)__float_as_uint(h.t) | (uint64_t)h.material << 32 | (uint64_t)h.face << 48 |
                       (uint64_t)h.shadow << 56;
    sw[3 * lane + 2] = (uint64_t)h.steps | (uint64_t)h.shadow_steps << 32;
  }
  __syncwarp();
  const uint32_t row_words = 3 * P.tile_w;
  uint64_t* base = reinterpret_cast<uint64_t*>(V.out);
  // Output in host memory, a CTA of four 8x4 tiles side by side, all inside
  // the image: after one barrier each warp writes one 32-pixel row of the
  // CTA (768 contiguous bytes, whole 128-byte lines when the row starts on
  // one), so no line crosses the CPU-GPU link in two pieces.  (Into device
  // memory the barrier costs more than it saves.)
  bool done = false;
  if (P.cta_rows && warps == 4 && P.tile_w == 8 && P.tile_h == 4 && (bid + 1) * 4 <= P.total_tiles) {
    const uint32_t x0 = px0 - 8u * (threadIdx.x >> 5);  // the CTA's first pixel column
    const bool ok = (tx & 3u) == (threadIdx.x >> 5) && px0 + 8 <= V.width && py0 + 4 <= V.height &&
                    ((reinterpret_cast<uintptr_t>(base) + (((uint64_t)py0 * V.width + x0) * 24)) & 15u) == 0 &&
                    (V.width & 1u) == 0;
    if (__syncthreads_and(ok)) {
      const uint32_t row = threadIdx.x >> 5;
      uint4* dst = reinterpret_cast<uint4*>(base + ((uint64_t)(py0 + row) * V.width + x0) * 3);
#pragma unroll
      for (int r = 0; r < 2; r++) {
        const uint32_t c = (uint32_t)lane + 32u * r;  // 16-byte chunk c of the row (48 in all)
        if (c < 48u) dst[c] = reinterpret_cast<const uint4*>(stage[c / 12u])[12u * row + c % 12u];
      }
      done = true;
    }
  }
  if (!done) {
    // a whole tile whose rows all start on 16 bytes goes out in 16-byte
    // stores, any other tile word by word
    const bool vec = ((reinterpret_cast<uintptr_t>(base) + (((uint64_t)py0 * V.width + px0) * 24)) & 15u) == 0 &&
                     (V.width & 1u) == 0 && (P.tile_w & 1u) == 0 && px0 + P.tile_w <= V.width &&
                     py0 + P.tile_h <= V.height;
    if (vec) {
      const uint32_t row_vecs = row_words / 2;
#pragma unroll
      for (int r = 0; r < 2; r++) {
        const uint32_t c = (uint32_t)lane + 32u * r;  // 16-byte chunk c of the tile (48 in all)
        if (c < 48u) {
          const uint32_t row = c / row_vecs, q = c % row_vecs;
          const uint4 v = reinterpret_cast<const uint4*>(sw)[c];
          reinterpret_cast<uint4*>(base + ((uint64_t)(py0 + row) * V.width + px0) * 3)[q] = v;
        }
      }
    } else {
#pragma unroll
      for (int r = 0; r < 3; r++) {
        const uint32_t c = (uint32_t)lane + 32u * r;  // word c of the tile: row c / row_words
        const uint32_t row = c / row_words, w = c % row_words;
        const uint32_t x = px0 + w / 3, y = py0 + row;
        if (x < V.width && y < V.height) base[((uint64_t)y * V.width + px0) * 3 + w] = sw[c];
      }
    }
  }
  if (kStats) {
    for (int k = 0; k < 4; k++) {
      const uint32_t tot = __reduce_add_sync(0xFFFFFFFFu, st[k]);
      if (lane == 0) atomicAdd(reinterpret_cast<unsigned long long*>(P.stats) + k, (unsigned long long)tot);
    }
  }
  if constexpr (kMode == kHashMode) {
    unsigned long long term = 0;
    uint32_t shadow = 0;
    if (px < V.width && py < V.height) {
      const uint64_t i = (uint64_t)py * V.width + px;
      const uint64_t w0 = sw[3 * lane], w1 = sw[3 * lane + 1], w2 = sw[3 * lane + 2];
      term = mix64(w0 ^ mix64(w1 ^ mix64(w2 ^ (i * 0x9E3779B97F4A7C15ull + 1ull))));
      shadow = (w2 >> 32) != 0;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) term += __shfl_down_sync(kFullMask, term, o);
    shadow = __reduce_add_sync(kFullMask, shadow);
    if (lane == 0) {
      const uint32_t slot = lo * kRayHashSlots + (bid & (kRayHashSlots - 1u));
      atomicAdd(P.hash + slot, term);
      if (shadow) atomicAdd(P.hash + kRayHashShadow + slot, (unsigned long long)shadow);
    }
  }
}

}  // namespace

size_t raymarch_view_table_bytes(uint32_t n_views) { return sizeof(RayView) * (size_t)n_views; }

// CTAs take their blocks in a strided order, b * 7919 mod blocks (a bijection
// unless blocks is a multiple of the prime 7919), so the cheap sky tiles and
// the expensive terrain tiles of a frame mix over the whole launch: the hit
// records leave at an even rate, which the CPU-GPU link needs when they are
// written to page-locked host memory (1080p end to end 0.48 -> 0.39 ms; the
// frame into device memory is unchanged).
static uint32_t block_order_mul(uint32_t blocks) { return blocks > 1 && blocks % 7919u ? 7919u : 0u; }

// Fills the host descriptors out[0 .. n) of views scenes/cams[0 .. n).  tiles
// and hits are running totals over all views of the launch (in: those of
// the views before these; out: including them).
static void fill_views(const meso_scene* const* scenes, const meso_camera* cams, uint32_t n, uint32_t tw, uint32_t th,
                       meso_hit* d_hits, meso_hit* const* view_out, RayView* out, uint64_t& tiles, uint64_t& hits) {
  for (uint32_t v = 0; v < n; v++) {
    const meso_scene* s = scenes[v];
    const meso_camera& c = cams[v];
    RayView& V = out[v];
    memset(&V, 0, sizeof(V));
    V.ptr = s->d_ptr;
    V.macro = s->d_macro;
    V.macro2 = s->d_macro2;
    V.macro3 = s->d_macro3;
    V.occ = s->d_occ;
    V.mat = s->d_mat;
    V.nx = s->nx;
    V.ny = s->ny;
    V.nz = s->nz;
    for (int a = 0; a < 3; a++) {
      V.cam_chunk[a] = c.origin_chunk[a];
      V.o[a] = c.origin_frac[a];
      V.fwd[a] = c.forward[a];
      V.right[a] = c.right[a];
      V.up[a] = c.up[a];
    }
    V.tan_half = c.tan_half_fov_y;
    V.aspect = (float)c.width / (float)c.height;  // IEEE conversions and division, as on the device
    V.width = c.width;
    V.height = c.height;
    V.tiles_x = (c.width + tw - 1) / tw;
    const uint32_t tiles_y = (c.height + th - 1) / th;
    V.tile_start = (uint32_t)tiles;
    V.out = view_out && view_out[v] ? view_out[v] : d_hits + hits;
    tiles += (uint64_t)V.tiles_x * tiles_y;
    hits += (uint64_t)c.width * c.height;
  }
}

}  // namespace meso

namespace meso {
namespace {

// Descriptors of up to kFillViews views, passed by value to the kernel that
// writes them into a device view table.  Kernel parameters are copied when
// the launch is issued (and kept by value in a captured graph node), so no
// host buffer has to outlive the call; 64 views are 9.5 KiB of parameters
// and of the caller's stack.
constexpr uint32_t kFillViews = 64;
struct ViewBatch {
  RayView v[kFillViews];
};
static_assert(sizeof(ViewBatch) <= 32000, "a view batch must fit the kernel parameter space");

__global__ void view_fill_kernel(const __grid_constant__ ViewBatch b, uint32_t n, RayView* dst) {
  const uint32_t words = n * (uint32_t)(sizeof(RayView) / 8);
  const uint64_t* src = reinterpret_cast<const uint64_t*>(b.v);
  uint64_t* d = reinterpret_cast<uint64_t*>(dst);
  for (uint32_t i = threadIdx.x; i < words; i += blockDim.x) d[i] = src[i];
}

}  // namespace

// Writes the descriptors of n_views views into the device table d_table,
// stream-ordered before the launch that reads it: one small kernel per 64
// views, the descriptors travelling as its parameters.  *tiles receives the
// total tiles of the views.
static meso_status stage_view_table(const meso_scene* const* scenes, const meso_camera* cams, uint32_t n_views,
                                    uint32_t tw, uint32_t th, meso_hit* d_hits, meso_hit* const* view_out,
                                    RayView* d_table, cudaStream_t st, uint64_t* tiles) {
  ViewBatch batch;
  uint64_t t = 0, hits = 0;
  for (uint32_t v0 = 0; v0 < n_views; v0 += kFillViews) {
    const uint32_t n = n_views - v0 < kFillViews ? n_views - v0 : kFillViews;
    fill_views(scenes + v0, cams + v0, n, tw, th, d_hits, view_out ? view_out + v0 : nullptr, batch.v, t, hits);
    view_fill_kernel<<<1, 128, 0, st>>>(batch, n, d_table + v0);
    MESO_CUDA_TRY(cudaGetLastError());
  }
  *tiles = t;
  return MESO_OK;
}

meso_status launch_raymarch(meso_ctx* ctx, const meso_scene* const* scenes, const meso_camera* cams,
                            uint32_t n_views, const float light[3], uint32_t flags, meso_hit* d_hits,
                            cudaStream_t st, void* d_view_table, size_t view_table_bytes, uint64_t* d_stats,
                            meso_hit* const* view_out, unsigned long long* d_hash, bool host_out) {
  if (!scenes || !cams || !d_hits) return fail(MESO_ERR_INVALID_ARG, "raymarch: null argument");
  if (n_views == 0) return MESO_OK;
  for (uint32_t v = 0; v < n_views; v++) {
    if (!scenes[v]) return fail(MESO_ERR_INVALID_ARG, "raymarch: null scene");
    if (cams[v].width == 0 || cams[v].height == 0 || cams[v].width > 16384 || cams[v].height > 16384)
      return fail(MESO_ERR_INVALID_ARG, "raymarch: image size out of range");
    if (view_out && (reinterpret_cast<uintptr_t>(view_out[v]) & 7u))
      return fail(MESO_ERR_INVALID_ARG, "raymarch: view output not 8-byte aligned");
  }
  if (d_hash && (d_stats || n_views > kRayHashViews))
    return fail(MESO_ERR_INVALID_ARG, "raymarch: checksums need at most 64 views and no statistics");
  if ((flags & MESO_RAY_SHADOW) && !light) return fail(MESO_ERR_INVALID_ARG, "raymarch: shadow without light");
  const uint32_t tw = ctx->tuning.ray_tile_w ? ctx->tuning.ray_tile_w : 8;
  if (32 % tw) return fail(MESO_ERR_INVALID_ARG, "raymarch: tile width must divide 32");
  const uint32_t th = 32 / tw;
  const uint32_t wpc = ctx->tuning.ray_warps_per_cta ? ctx->tuning.ray_warps_per_cta : 4;
  RayParams P;
  memset(&P, 0, sizeof(P));
  P.n_views = n_views;
  P.tile_w = tw;
  P.tile_h = th;
  P.shadow = (flags & MESO_RAY_SHADOW) ? 1u : 0u;
  if (light)
    for (int a = 0; a < 3; a++) {
      P.light[a] = light[a];
      P.inv_light[a] = light[a] != 0.0f ? 1.0f / light[a] : 0.0f;  // IEEE division, as __fdiv_rn
    }
  P.stats = d_stats;
  P.hash = d_hash;
  P.cta_rows = host_out ? 1u : 0u;
  static InlineViews empty_views;  // zero-initialised
  uint64_t tiles;
  if (n_views <= (uint32_t)kInlineViews) {
    InlineViews iv;
    tiles = 0;
    uint64_t hits = 0;
    fill_views(scenes, cams, n_views, tw, th, d_hits, view_out, iv.v, tiles, hits);
    if (tiles >= (1ull << 31)) return fail(MESO_ERR_INVALID_ARG, "raymarch: too many tiles");
    P.total_tiles = (uint32_t)tiles;
    const uint32_t blocks = (uint32_t)((tiles + wpc - 1) / wpc);
    P.order_mul = block_order_mul(blocks);
    if (d_stats) raymarch_kernel<true, kStatsMode><<<blocks, wpc * 32, 0, st>>>(P, iv);
    else if (d_hash) raymarch_kernel<true, kHashMode><<<blocks, wpc * 32, 0, st>>>(P, iv);
    else raymarch_kernel<true, kPlain><<<blocks, wpc * 32, 0, st>>>(P, iv);
  } else {
    if (!d_view_table || view_table_bytes < raymarch_view_table_bytes(n_views))
      return fail(MESO_ERR_INVALID_ARG, "raymarch: view table too small");
    MESO_TRY(stage_view_table(scenes, cams, n_views, tw, th, d_hits, view_out, static_cast<RayView*>(d_view_table),
                              st, &tiles));
    if (tiles >= (1ull << 31)) return fail(MESO_ERR_INVALID_ARG, "raymarch: too many tiles");
    P.total_tiles = (uint32_t)tiles;
    P.table = static_cast<const RayView*>(d_view_table);
    const uint32_t blocks = (uint32_t)((tiles + wpc - 1) / wpc);
    P.order_mul = block_order_mul(blocks);
    if (d_stats) raymarch_kernel<false, kStatsMode><<<blocks, wpc * 32, 0, st>>>(P, empty_views);
    else if (d_hash) raymarch_kernel<false, kHashMode><<<blocks, wpc * 32, 0, st>>>(P, empty_views);
    else raymarch_kernel<false, kPlain><<<blocks, wpc * 32, 0, st>>>(P, empty_views);
  }
  ctx->launches.fetch_add(1);
  MESO_CUDA_TRY(cudaGetLastError());
  return MESO_OK;
}

}  // namespace meso

// ---------------------------------------------------------------------------
// Multi-view raymarch that allocates nothing.
//
// meso_raymarch stages the descriptor table of more than 32 views in device
// memory it allocates per call.  Some callers cannot allocate device memory
// at that point: a frame loop running on a fixed device-memory budget that
// must not allocate mid-frame (an allocation can synchronise the device and
// stall the frame), or a host application whose own memory manager owns all
// device memory.  This entry point keeps the table in a fixed file-scope
// device array instead; the descriptors reach it as kernel parameters, 64
// views at a time, through a 9.5 KiB batch on the caller's stack.
//
// Limits and behaviour:
//  - at most kNoAllocViews (512) views per call; more is rejected with
//    MESO_ERR_INVALID_ARG;
//  - the array (512 x 152 B = 76 KiB) stays resident on every device that
//    loads the library until the process exits;
//  - the calling thread's current device must be the context's device;
//  - the first call on a device looks up the array's device address (with
//    that device current) and caches it; make that first call before any
//    stream capture;
//  - every call reuses the same array and overwrites the entries it uses, so
//    calls whose kernels overlap on the GPU race on it: issue them on one
//    stream, or order them with events.
namespace meso {
namespace {

constexpr uint32_t kNoAllocViews = 512;
static_assert(sizeof(RayView) == 152, "the documented size of the fixed view table is 512 x 152 bytes");
static __device__ __align__(256) unsigned char g_noalloc_views[kNoAllocViews * sizeof(RayView)];

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[64] = {};

// Device address of g_noalloc_views on `device` (looked up once per device;
// `device` is current when this is called).
meso_status noalloc_table(int device, void** out) {
  if (device < 0 || device >= 64) return fail(MESO_ERR_INVALID_ARG, "raymarch_noalloc: device ordinal >= 64");
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_views);
    if (e != cudaSuccess) return cuda_fail(e, "raymarch_noalloc: cudaGetSymbolAddress");
    g_noalloc_ptr[device] = p;
  }
  *out = g_noalloc_ptr[device];
  return MESO_OK;
}

}  // namespace
}  // namespace meso

extern "C" meso_status meso_raymarch_noalloc(meso_ctx* ctx, const meso_scene* const* scenes,
                                             const meso_camera* h_cams, uint32_t n_views, const float light[3],
                                             uint32_t flags, meso_hit* d_hits, void* stream) {
  using namespace meso;
  if (!ctx || !scenes || !h_cams || !d_hits) return fail(MESO_ERR_INVALID_ARG, "raymarch_noalloc: null argument");
  if (n_views > kNoAllocViews)
    return fail(MESO_ERR_INVALID_ARG, "raymarch_noalloc: at most 512 views per call (fixed device view table)");
  if (n_views == 0) return MESO_OK;
  for (uint32_t v = 0; v < n_views; v++) {
    if (!scenes[v]) return fail(MESO_ERR_INVALID_ARG, "raymarch_noalloc: null scene");
    if (h_cams[v].width == 0 || h_cams[v].height == 0 || h_cams[v].width > 16384 || h_cams[v].height > 16384)
      return fail(MESO_ERR_INVALID_ARG, "raymarch_noalloc: image size out of range");
  }
  if ((flags & MESO_RAY_SHADOW) && !light) return fail(MESO_ERR_INVALID_ARG, "raymarch_noalloc: shadow without light");
  const uint32_t tw = ctx->tuning.ray_tile_w ? ctx->tuning.ray_tile_w : 8;
  if (32 % tw) return fail(MESO_ERR_INVALID_ARG, "raymarch_noalloc: tile width must divide 32");
  const uint32_t th = 32 / tw;
  const uint32_t wpc = ctx->tuning.ray_warps_per_cta ? ctx->tuning.ray_warps_per_cta : 4;
  int cur = -1;
  MESO_CUDA_TRY(cudaGetDevice(&cur));
  if (cur != ctx->device)
    return fail(MESO_ERR_INVALID_ARG, "raymarch_noalloc: the current device is not the context's device");
  void* table = nullptr;
  MESO_TRY(noalloc_table(ctx->device, &table));
  // the same validation as meso_raymarch, before any work is issued
  uint64_t tiles = 0;
  for (uint32_t v = 0; v < n_views; v++)
    tiles += (uint64_t)((h_cams[v].width + tw - 1) / tw) * ((h_cams[v].height + th - 1) / th);
  if (tiles >= (1ull << 31)) return fail(MESO_ERR_INVALID_ARG, "raymarch_noalloc: too many tiles");
  RayParams P;
  memset(&P, 0, sizeof(P));
  P.table = static_cast<const RayView*>(table);
  P.n_views = n_views;
  P.total_tiles = (uint32_t)tiles;
  P.tile_w = tw;
  P.tile_h = th;
  P.shadow = (flags & MESO_RAY_SHADOW) ? 1u : 0u;
  if (light)
    for (int a = 0; a < 3; a++) {
      P.light[a] = light[a];
      P.inv_light[a] = light[a] != 0.0f ? 1.0f / light[a] : 0.0f;  // IEEE division, as __fdiv_rn
    }
  const cudaStream_t st = pick_stream(ctx, stream);
  MESO_TRY(stage_view_table(scenes, h_cams, n_views, tw, th, d_hits, nullptr, static_cast<RayView*>(table), st,
                            &tiles));
  static InlineViews unused_inline;  // zero-initialised; the table path does not read it
  const uint32_t blocks = (uint32_t)((tiles + wpc - 1) / wpc);
  P.order_mul = block_order_mul(blocks);
  raymarch_kernel<false, kPlain><<<blocks, wpc * 32, 0, st>>>(P, unused_inline);
  ctx->launches.fetch_add(1);
  MESO_CUDA_TRY(cudaGetLastError());
  return MESO_OK;
}
