// mesh.cu -- greedy chunk meshing on sm_103a.
//
// Replaces the reference's per-chunk host work: the 26-neighbour erosion cull
// (Runtimes/Voxel/Occupancy/BinaryOccupancyVolume.h:76-99, run from
// Runtimes/Voxel/Chunk/Chunk.h:73-100) and the one-instance-per-visible-block
// emission of FChunkPool::PushToBlockPool (Runtimes/Voxel/Chunk/ChunkPool.h:381-445),
// dispatched 8 chunks per host task by FChunkManage::MultiThreadGeneratorBatched
// (Runtimes/Voxel/Chunk/ChunkManager.h:183-210).  Here a persistent kernel
// pulls chunks from a device ticket queue and emits greedy quads.
//
// Two CTAs of 16 warps share each SM (64 registers per thread), each meshing
// its own chunk, so one CTA's barrier-separated phases overlap the other's
// work; the kernel is latency bound and 32 resident warps hide more of it
// than 16 or 24 did.  Per chunk:
//  1. staging: the 32^3 materials arrive in shared memory asynchronously
//     (TMA: one bulk copy per chunk of a chunk array, one 3-D tensor box per
//     chunk of a dense grid; for a brick map 16-byte copies of the occupied
//     bricks by the whole CTA, after the chunk has been picked out of a
//     ticket of chunks tested together against the scene's cell map); the
//     one-voxel occupancy halo is read with plain loads while it lands;
//  2. masks: lanes = x; every row (y,z) becomes bit-packed words with warp
//     ballots: occupancy and material-equality with the -x, -y and -z
//     neighbour, plus warp-transposed copies (bits over y) for the X faces;
//     face masks occ & ~shift(occ) are recomputed from these where needed;
//  3. faces whose quad cannot depend on the scan order are peeled off
//     first: isolated faces (no same-material face neighbour in their plane)
//     become 1x1 quads through a warp-balanced expansion with one output
//     reservation per warp and chunk, and two-face components become 2x1 or
//     1x2 quads at the start of their slice's greedy;
//  4. greedy: warp = slice with non-isolated faces, lane = row; rows are
//     scanned with run-length bit tricks (Lysenko's order: first unconsumed
//     face, widen along u while the material matches, grow along v while the
//     whole run matches); quads are staged per warp in shared memory and
//     appended to global memory with one atomic per 64 quads.
#include <cudaTypedefs.h>

#include <cstdio>
#include <cstring>

#include "meso_internal.h"

namespace meso {
namespace {

using namespace ::meso::dev;

constexpr int kThreads = 512;
constexpr int kWarps = kThreads / 32;
// Warps w and w + 8 form a pair that shares rows (and slabs) 4(w mod 8) ..
// 4(w mod 8) + 3: in the mask pass each builds half of the slabs' rows, in
// the isolated-face passes each takes three of the six face directions.
constexpr int kGroups = 12;  // word groups (direction, row) per warp: 4 rows x 3 directions
static_assert(kWarps == 16, "eight warp pairs of 4 rows each");
constexpr int kS = 33;               // padded row stride of 32x32 word arrays
constexpr int kArr = 32 * kS;
constexpr int kQBuf = 64;            // staged quads per warp
constexpr int kBrickSlot = 1040;     // bytes per staged brick (bank-spread padding)
constexpr uint32_t kFull = 0xFFFFFFFFu;
constexpr uint64_t kWaitLimitNs = 2000000000ull;

// Shared memory of one CTA: these arrays, then the staged materials of the
// chunk (KindTraits::kMatBytes, 128-byte aligned).
struct __align__(128) MeshSmem {
  uint32_t occ[kArr];                     // occupancy, bits over x, [z][y]
  uint32_t occt[kArr];                    // occupancy, bits over y, [z][x]
  uint32_t ex[kArr], ey[kArr], ez[kArr];  // equality with -x / -y / -z neighbour, bits over x, [z][y]
  uint32_t eyt[kArr], ezt[kArr];          // equality with -y / -z neighbour, bits over y, [z][x]
  uint32_t halo[6][32];                   // -X,+X: bits y by z; -Y,+Y: bits x by z; -Z,+Z: bits x by y
  uint64_t qbuf[kWarps][kQBuf];           // staged greedy quads per warp
  uint32_t rest_slices[6];                // per direction: bit s = slice s holds non-isolated faces
  uint64_t bar;
  int32_t chunk;
  int32_t valid;
  int32_t coord[3];
  uint32_t chunk_quads;
  uint32_t task_next;                     // dynamic task counter of the greedy
  uint32_t any_solid;
  uint32_t bptr[64];  // brick maps: the chunk's 64 brick pointers
};

struct MeshParams {
  const uint8_t* data;
  int32_t nx, ny, nz;
  const uint32_t* bptr;
  const uint64_t* bocc;
  const uint16_t* bmat;
  const uint8_t* bcell;  // per 4x4x4-brick cell (one chunk): nonzero iff a brick of it is occupied
  int32_t bx, by, bz;
  const int32_t* coords;
  uint32_t n_chunks;
  uint32_t chunk_id_base;
  uint64_t* quads;
  uint64_t cap;
  unsigned long long* count;
  uint32_t* chunk_counts;
  uint32_t* ticket;
  uint32_t* err;
  uint32_t per_ticket;
  int32_t use_queue;
  uint32_t perm_mul;  // brick maps: ticket t takes list entry (t * perm_mul) mod n_chunks
};

// Per source kind: halo reads, addressing, element size, the staged bytes of
// one chunk, and the CTAs per SM (two of 16 warps: the register file allows
// no more, and 16-bit chunks fill the shared memory of two).
template <int KIND>
struct KindTraits;
template <int KIND>
struct KindBase {
  static constexpr bool kHalo = KIND != MESO_SRC_CHUNKS_U16 && KIND != MESO_SRC_CHUNKS_U8;
  static constexpr bool kGrid = KIND == MESO_SRC_GRID_U8 || KIND == MESO_SRC_GRID_U16;
  static constexpr bool kBrick = KIND == MESO_SRC_BRICKMAP;
  static constexpr int kElem = KIND == MESO_SRC_CHUNKS_U8 || KIND == MESO_SRC_GRID_U8 ? 1 : 2;
  static constexpr int kMatBytes = kBrick ? 64 * kBrickSlot : 32768 * kElem;
  static constexpr int kCtasPerSm = 2;
  static_assert(sizeof(MeshSmem) + kMatBytes + 128 + 1024 <= 228 * 1024 / kCtasPerSm,
                "the mesher's CTAs per SM must fit the shared memory");
};
template <>
struct KindTraits<MESO_SRC_CHUNKS_U16> : KindBase<MESO_SRC_CHUNKS_U16> {};
template <>
struct KindTraits<MESO_SRC_CHUNKS_U8> : KindBase<MESO_SRC_CHUNKS_U8> {};
template <>
struct KindTraits<MESO_SRC_GRID_U8> : KindBase<MESO_SRC_GRID_U8> {};
template <>
struct KindTraits<MESO_SRC_GRID_U16> : KindBase<MESO_SRC_GRID_U16> {};
template <>
struct KindTraits<MESO_SRC_BRICKMAP> : KindBase<MESO_SRC_BRICKMAP> {};

template <int KIND>
__device__ __forceinline__ uint32_t load_mat(const uint8_t* buf, int x, int y, int z) {
  using T = KindTraits<KIND>;
  if constexpr (T::kBrick) {
    const int b = (x >> 3) + 4 * (y >> 3) + 16 * (z >> 3);
    return reinterpret_cast<const uint16_t*>(buf + b * kBrickSlot)[(x & 7) + 8 * (y & 7) + 64 * (z & 7)];
  } else if constexpr (T::kElem == 2) {
    return reinterpret_cast<const uint16_t*>(buf)[(z * 32 + y) * 32 + x];
  } else {
    return buf[(z * 32 + y) * 32 + x];
  }
}

// Material at chunk-local linear index lin = x + 32 y + 1024 z.
template <int KIND>
__device__ __forceinline__ uint32_t load_mat_lin(const uint8_t* buf, uint32_t lin) {
  using T = KindTraits<KIND>;
  if constexpr (T::kBrick) {
    return load_mat<KIND>(buf, (int)(lin & 31u), (int)((lin >> 5) & 31u), (int)(lin >> 10));
  } else if constexpr (T::kElem == 2) {
    return reinterpret_cast<const uint16_t*>(buf)[lin];
  } else {
    return buf[lin];
  }
}

// True iff the 8 rows y0..y0+7 (y0 % 8 == 0) of slab z are all empty: one
// 16-byte (8-byte for uint8) shared load per lane covers the 256 voxels.
template <int KIND>
__device__ __forceinline__ bool rows8_empty(const uint8_t* buf, int y0, int z, int lane) {
  using T = KindTraits<KIND>;
  bool nz;
  if constexpr (T::kBrick) {
    const int b = (lane >> 3) + 4 * (y0 >> 3) + 16 * (z >> 3);
    const uint4 w = *reinterpret_cast<const uint4*>(buf + b * kBrickSlot + 128 * (z & 7) + 16 * (lane & 7));
    nz = (w.x | w.y | w.z | w.w) != 0;
  } else if constexpr (T::kElem == 2) {
    const uint4 w = *reinterpret_cast<const uint4*>(buf + (z * 32 + y0) * 64 + 16 * lane);
    nz = (w.x | w.y | w.z | w.w) != 0;
  } else {
    const uint2 w = *reinterpret_cast<const uint2*>(buf + (z * 32 + y0) * 32 + 8 * lane);
    nz = (w.x | w.y) != 0;
  }
  return !__any_sync(kFull, nz);
}

// Occupancy (material != 0) of a global voxel for halo reads; 0 outside.
template <int KIND>
__device__ __forceinline__ uint32_t global_solid(const MeshParams& p, int gx, int gy, int gz) {
  using T = KindTraits<KIND>;
  if (gx < 0 || gy < 0 || gz < 0) return 0;
  if constexpr (T::kBrick) {
    if (gx >= p.bx * 8 || gy >= p.by * 8 || gz >= p.bz * 8) return 0;
    const uint32_t ptr = __ldg(p.bptr + (gx >> 3) + (size_t)p.bx * ((gy >> 3) + (size_t)p.by * (gz >> 3)));
    if (ptr == MESO_EMPTY_BRICK) return 0;
    const uint64_t w = __ldg(p.bocc + (size_t)ptr * 8 + (gz & 7));
    return (uint32_t)(w >> ((gx & 7) + 8 * (gy & 7))) & 1u;
  } else {
    if (gx >= p.nx || gy >= p.ny || gz >= p.nz) return 0;
    const size_t i = (size_t)gx + (size_t)p.nx * ((size_t)gy + (size_t)p.ny * (size_t)gz);
    if constexpr (T::kElem == 2) return __ldg(reinterpret_cast<const uint16_t*>(p.data) + i) != 0;
    else return __ldg(p.data + i) != 0;
  }
}

// Producer side: called by warp 0 (all lanes).  Takes the next chunk off the
// queue and starts its copy into the staging buffer.  Lane 0 holds the queue
// state: [cur, end) is the current ticket's range and `pending` the start of
// the next ticket, requested one ticket ahead so the atomic's latency is
// hidden behind a chunk's work.
//
// Brick maps take a ticket of per_ticket (<= 32) list entries at a time, one
// per lane, through the bijection t -> (t * perm_mul) mod n_chunks so that a
// ticket samples the whole list (runs of neighbouring chunks are all air or
// all terrain), and test them together against the scene's cell map: a chunk
// with no occupied brick has no solid voxel and so no face, and is counted
// (0 quads) and passed over here, without a round trip through the CTA.
// bc is this lane's entry of the current ticket, bmask the lanes whose entry
// is still to be meshed (an entry with an invalid coordinate is meshed, to
// be flagged there).
template <int KIND>
__device__ __forceinline__ void issue_chunk(MeshSmem& sm, uint8_t* dst, const MeshParams& p, const CUtensorMap* tmap,
                                            int lane, uint32_t& cur, uint32_t& end, uint32_t& pending, int& bc,
                                            uint32_t& bmask) {
  using T = KindTraits<KIND>;
  int c = -1;
  int bx3[3] = {0, 0, 0};
  bool have_xyz = false;
  if constexpr (T::kBrick) {
    if (p.use_queue) {
      const int MX = p.bx >> 2, MY = p.by >> 2, MZ = p.bz >> 2;
      for (;;) {
        if (bmask == 0) {
          uint32_t t0 = 0;
          if (lane == 0) t0 = atomicAdd(p.ticket, p.per_ticket);
          t0 = __shfl_sync(kFull, t0, 0);
          if (t0 >= p.n_chunks) break;
          const uint32_t t = t0 + (uint32_t)lane;
          bool need = false;
          bc = -1;
          if ((uint32_t)lane < p.per_ticket && t < p.n_chunks) {
            bc = (int)(((uint64_t)t * p.perm_mul) % p.n_chunks);
            const int x = p.coords[3 * bc], y = p.coords[3 * bc + 1], z = p.coords[3 * bc + 2];
            const bool ok = x >= 0 && y >= 0 && z >= 0 && x < MX && y < MY && z < MZ;
            need = !ok || __ldg(p.bcell + x + (size_t)MX * (y + (size_t)MY * z)) != 0;
            if (!need && p.chunk_counts) p.chunk_counts[bc] = 0;
          }
          bmask = __ballot_sync(kFull, need);
          continue;
        }
        const int l = __ffs(bmask) - 1;
        bmask &= bmask - 1u;
        c = __shfl_sync(kFull, bc, l);
        break;
      }
      if (lane == 0) sm.chunk = c;
      if (c < 0) return;
      have_xyz = true;
      if (lane == 0) {
        bx3[0] = p.coords[3 * c];
        bx3[1] = p.coords[3 * c + 1];
        bx3[2] = p.coords[3 * c + 2];
      }
    }
  }
  if (!have_xyz && lane == 0) {
    if (p.use_queue) {
      if (cur >= end) {
        cur = pending;
        end = cur + p.per_ticket;
        pending = atomicAdd(p.ticket, p.per_ticket);
      }
      if (cur < p.n_chunks) c = (int)cur++;
    } else {
      if (cur < p.n_chunks) {
        c = (int)cur;
        cur += gridDim.x;
      }
    }
  }
  if (!have_xyz) {
    c = __shfl_sync(kFull, c, 0);
    if (lane == 0) sm.chunk = c;
    if (c < 0) return;
  }
  uint64_t* bar = &sm.bar;
  if constexpr (!T::kGrid && !T::kBrick) {
    if (lane == 0) {
      // with an index list, p.nx is the number of chunks in the array
      const uint32_t idx = p.coords ? (uint32_t)p.coords[c] : (uint32_t)c;
      const bool ok = !p.coords || idx < (uint32_t)p.nx;
      sm.valid = ok ? 1 : 0;
      if (!ok) {
        atomicOr(p.err, ERR_BAD_INPUT);
        mbar_arrive_expect_tx(bar, 0);
      } else {
        const uint32_t bytes = 32768u * T::kElem;
        const uint8_t* src = p.data + (size_t)idx * bytes;
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(bar, bytes);
        for (uint32_t off = 0; off < bytes; off += 16384u) bulk_g2s(dst + off, src + off, 16384u, bar);
      }
    }
  } else {
    int cx = bx3[0], cy = bx3[1], cz = bx3[2];
    if (lane == 0 && !have_xyz) {
      cx = p.coords[3 * c];
      cy = p.coords[3 * c + 1];
      cz = p.coords[3 * c + 2];
    }
    cx = __shfl_sync(kFull, cx, 0);
    cy = __shfl_sync(kFull, cy, 0);
    cz = __shfl_sync(kFull, cz, 0);
    int lim_x, lim_y, lim_z;
    if constexpr (T::kBrick) {
      lim_x = p.bx / 4;
      lim_y = p.by / 4;
      lim_z = p.bz / 4;
    } else {
      lim_x = p.nx / 32;
      lim_y = p.ny / 32;
      lim_z = p.nz / 32;
    }
    const bool ok = cx >= 0 && cy >= 0 && cz >= 0 && cx < lim_x && cy < lim_y && cz < lim_z;
    if (lane == 0) {
      sm.coord[0] = cx;
      sm.coord[1] = cy;
      sm.coord[2] = cz;
      sm.valid = ok ? 1 : 0;
    }
    if (!ok) {
      if (lane == 0) {
        atomicOr(p.err, ERR_BAD_INPUT);
        mbar_arrive_expect_tx(bar, 0);
      }
      return;
    }
    if constexpr (T::kGrid) {
      if (lane == 0) {
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(bar, 32768u * T::kElem);
        tma_load_3d(dst, tmap, cx * 32, cy * 32, cz * 32, bar);
      }
    } else {
      // 64 bricks, two per lane
      uint32_t ptrs[2];
      for (int k = 0; k < 2; k++) {
        const int b = lane + 32 * k;
        const int gx = cx * 4 + (b & 3), gy = cy * 4 + ((b >> 2) & 3), gz = cz * 4 + (b >> 4);
        ptrs[k] = __ldg(p.bptr + gx + (size_t)p.bx * (gy + (size_t)p.by * gz));
      }
      const uint32_t n_full = __popc(__ballot_sync(kFull, ptrs[0] != MESO_EMPTY_BRICK)) +
                              __popc(__ballot_sync(kFull, ptrs[1] != MESO_EMPTY_BRICK));
      // the whole CTA copies the bricks' materials after the barrier (16-byte
      // asynchronous copies); the mbarrier phase completes with no bytes
      sm.bptr[lane] = ptrs[0];
      sm.bptr[lane + 32] = ptrs[1];
      if (lane == 0) {
        mbar_arrive_expect_tx(bar, 0);
        // no occupied brick: no solid voxel, so no face and nothing to stage
        if (n_full == 0) sm.valid = 2;
      }
      (void)dst;  // staged after the CTA barrier (mesh_kernel)
    }
  }
}

// The chunk the next issue_chunk will take (lane 0 of warp 0), so its data
// can be prefetched into L2 while this chunk is meshed.  Only the index (and
// for grid sources the coordinates) is loaded here; prefetch_chunk uses it
// later, after the load has landed.  a < 0: nothing to prefetch.
template <int KIND>
__device__ __forceinline__ void next_chunk(const MeshParams& p, uint32_t cur, uint32_t end, uint32_t pending,
                                           int32_t& a, int32_t& b, int32_t& c) {
  using T = KindTraits<KIND>;
  a = -1;
  const uint32_t n = p.use_queue ? (cur < end ? cur : pending) : cur;
  if (n >= p.n_chunks || T::kBrick) return;
  if constexpr (T::kGrid) {
    a = p.coords[3 * n];
    b = p.coords[3 * n + 1];
    c = p.coords[3 * n + 2];
  } else {
    a = p.coords ? p.coords[n] : (int32_t)n;
  }
}

template <int KIND>
__device__ __forceinline__ void prefetch_chunk(const MeshParams& p, const CUtensorMap* tmap, int32_t a, int32_t b,
                                               int32_t c) {
  using T = KindTraits<KIND>;
  if (a < 0) return;
  if constexpr (T::kGrid) {
    if (b >= 0 && c >= 0 && a < p.nx / 32 && b < p.ny / 32 && c < p.nz / 32) tma_prefetch_3d(tmap, a * 32, b * 32, c * 32);
  } else if constexpr (!T::kBrick) {
    if (!p.coords || a < p.nx) bulk_prefetch_l2(p.data + (size_t)a * 32768u * T::kElem, 32768u * T::kElem);
  }
}

// The one-voxel occupancy halo around the chunk: 6 faces x 32 rows, a row
// per ballot.  Each warp reads its 12 rows' voxels first (for a brick map a
// pointer load and a dependent occupancy load each) so all of them are in
// flight together, then ballots them.
template <int KIND>
__device__ __forceinline__ void compute_halos(MeshSmem& sm, const MeshParams& p, int warp, int lane) {
  constexpr int kPer = 6 * 32 / kWarps;
  static_assert(kPer * kWarps == 6 * 32, "halo rows split evenly over the warps");
  const int X = sm.coord[0] * 32, Y = sm.coord[1] * 32, Z = sm.coord[2] * 32;
  uint32_t solid[kPer];
#pragma unroll
  for (int i = 0; i < kPer; i++) {
    const int wi = warp + kWarps * i;
    const int f = wi >> 5, k = wi & 31;
    int gx, gy, gz;
    switch (f) {
      case 0: gx = X - 1; gy = Y + lane; gz = Z + k; break;
      case 1: gx = X + 32; gy = Y + lane; gz = Z + k; break;
      case 2: gx = X + lane; gy = Y - 1; gz = Z + k; break;
      case 3: gx = X + lane; gy = Y + 32; gz = Z + k; break;
      case 4: gx = X + lane; gy = Y + k; gz = Z - 1; break;
      default: gx = X + lane; gy = Y + k; gz = Z + 32; break;
    }
    solid[i] = global_solid<KIND>(p, gx, gy, gz);
  }
#pragma unroll
  for (int i = 0; i < kPer; i++) {
    const int wi = warp + kWarps * i;
    const uint32_t w = __ballot_sync(kFull, solid[i] != 0);
    if (lane == 0) sm.halo[wi >> 5][wi & 31] = w;
  }
}

// In-register 32x32 bit transpose across a warp: lane r holds row r (bit c =
// element (r, c)); afterwards lane c holds column c (bit r).  Five butterfly
// stages swap the off-diagonal blocks of size 16, 8, 4, 2, 1.
__device__ __forceinline__ uint32_t transpose32(uint32_t x, int lane) {
#pragma unroll
  for (int j = 16; j >= 1; j >>= 1) {
    const uint32_t lo = j == 16 ? 0x0000FFFFu : j == 8 ? 0x00FF00FFu : j == 4 ? 0x0F0F0F0Fu : j == 2 ? 0x33333333u
                                                                                                      : 0x55555555u;
    const uint32_t t = __shfl_xor_sync(kFull, x, j);
    x = (lane & j) ? ((x & ~lo) | ((t & ~lo) >> j)) : ((x & lo) | ((t & lo) << j));
  }
  return x;
}

// Array addressing of direction d: (slice s, row v) -> word offset.
__device__ __forceinline__ int word_off(int d, int s, int v) { return d < 4 ? v * kS + s : s * kS + v; }

// Origin voxel of a face at (dir d, slice s, column u, row v).
__device__ __forceinline__ void face_xyz(int d, int s, int u, int v, int& x, int& y, int& z) {
  if (d < 2) { x = s; y = u; z = v; }
  else if (d < 4) { x = u; y = s; z = v; }
  else { x = u; y = v; z = s; }
}

// In-plane equality arrays of direction d: E along u, V along v.
__device__ __forceinline__ const uint32_t* e_arr(const MeshSmem& sm, int d) { return d < 2 ? sm.eyt : sm.ex; }
__device__ __forceinline__ const uint32_t* v_arr(const MeshSmem& sm, int d) {
  return d < 2 ? sm.ezt : (d < 4 ? sm.ez : sm.ey);
}

// Face word of direction d, row v, for the slice s = lane (all lanes call):
// the occupancy word of the slice minus that of the next slice along the
// face normal, taken from the neighbouring lane or the halo.
__device__ __forceinline__ uint32_t face_row(const MeshSmem& sm, int d, int v, int lane) {
  uint32_t c, hi, lo;
  if (d < 2) {
    c = sm.occt[v * kS + lane];
    hi = sm.halo[1][v];
    lo = sm.halo[0][v];
  } else if (d < 4) {
    c = sm.occ[v * kS + lane];
    hi = sm.halo[3][v];
    lo = sm.halo[2][v];
  } else {
    c = sm.occ[lane * kS + v];
    hi = sm.halo[5][v];
    lo = sm.halo[4][v];
  }
  uint32_t n;
  if ((d & 1) == 0) {
    n = __shfl_down_sync(kFull, c, 1);
    if (lane == 31) n = hi;
  } else {
    n = __shfl_up_sync(kFull, c, 1);
    if (lane == 0) n = lo;
  }
  return c & ~n;
}

// Face word of direction d, slice s, for the row v = r (lanes = rows).
__device__ __forceinline__ uint32_t face_col(const MeshSmem& sm, int d, int s, int r) {
  const bool pos = (d & 1) == 0;
  const int sn = pos ? s + 1 : s - 1;
  const bool edge = pos ? s == 31 : s == 0;
  // halo[d ^ 1] is the layer beyond the chunk on the side the face points to
  if (d < 2) return sm.occt[r * kS + s] & ~(edge ? sm.halo[d ^ 1][r] : sm.occt[r * kS + sn]);
  if (d < 4) return sm.occ[r * kS + s] & ~(edge ? sm.halo[d ^ 1][r] : sm.occ[r * kS + sn]);
  return sm.occ[s * kS + r] & ~(edge ? sm.halo[d ^ 1][r] : sm.occ[sn * kS + r]);
}

// Faces of a word with a same-material face neighbour in the plane: f the
// faces of the row, fu / fd those of rows v-1 / v+1, e equality with the -u
// neighbour, vv / vd equality of this row / of row v+1 with the row above.
__device__ __forceinline__ uint32_t isolated(uint32_t f, uint32_t fu, uint32_t fd, uint32_t e, uint32_t vv,
                                             uint32_t vd) {
  const uint32_t left = f & e & (f << 1);
  return f & ~(left | (left >> 1) | (f & vv & fu) | (f & vd & fd));
}

// Position of the (r+1)-th set bit of w (r < popc(w)): halving on popcounts.
__device__ __forceinline__ uint32_t select_bit(uint32_t w, uint32_t r) {
  uint32_t pos = 0, c;
  c = __popc(w & 0xFFFFu);
  if (r >= c) { r -= c; w >>= 16; pos = 16; }
  c = __popc(w & 0xFFu);
  if (r >= c) { r -= c; w >>= 8; pos += 8; }
  c = __popc(w & 0xFu);
  if (r >= c) { r -= c; w >>= 4; pos += 4; }
  c = __popc(w & 0x3u);
  if (r >= c) { r -= c; w >>= 2; pos += 2; }
  return pos + (r >= (w & 1u) ? 1u : 0u);
}

// Appends the warp's staged quads to the output (one atomic per flush).
__device__ __forceinline__ void flush_warp(MeshSmem& sm, int warp, const MeshParams& p, int lane, uint32_t cnt) {
  __syncwarp();
  unsigned long long base = 0;
  if (lane == 0 && cnt) base = atomicAdd(p.count, (unsigned long long)cnt);
  base = __shfl_sync(kFull, base, 0);
  for (uint32_t i = lane; i < cnt; i += 32) {
    const unsigned long long idx = base + i;
    if (idx < p.cap) p.quads[idx] = sm.qbuf[warp][i];
  }
  __syncwarp();
}

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Barrier of the warp pair that shares row group g (ids 1..8; 0 is __syncthreads).
__device__ __forceinline__ void pair_sync(int g) {
  asm volatile("bar.sync %0, 64;" ::"r"(1 + g) : "memory");
}

// Isolated faces of the three directions DB .. DB+2 for the rows v0 .. v0+3
// (lane = slice); see pass 2 in the kernel.
template <int DB>
__device__ __forceinline__ void isolated_rows(MeshSmem& sm, int v0, int lane, uint32_t (&isow)[kGroups],
                                              uint32_t& lane_iso) {
#pragma unroll
  for (int dd = 0; dd < 3; dd++) {
    const int d = DB + dd;
    uint32_t fu = v0 > 0 ? face_row(sm, d, v0 - 1, lane) : 0u;
    uint32_t fv = face_row(sm, d, v0, lane);
    uint32_t vv = v_arr(sm, d)[word_off(d, lane, v0)];
    uint32_t rest = 0;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int v = v0 + q;
      const bool last = q == 3 && v0 == 28;
      const uint32_t fd = last ? 0u : face_row(sm, d, v + 1, lane);
      const uint32_t vd = last ? 0u : v_arr(sm, d)[word_off(d, lane, v + 1)];
      const uint32_t w = isolated(fv, fu, fd, e_arr(sm, d)[word_off(d, lane, v)], vv, vd);
      isow[4 * dd + q] = w;
      lane_iso += __popc(w);
      rest |= fv & ~w;
      fu = fv;
      fv = fd;
      vv = vd;
    }
    const uint32_t m = __ballot_sync(kFull, rest != 0u);
    if (lane == 0 && m) atomicOr(&sm.rest_slices[d], m);
  }
}

template <int KIND>
__global__ void __launch_bounds__(kThreads, KindTraits<KIND>::kCtasPerSm)
    mesh_kernel(const MeshParams p, const __grid_constant__ CUtensorMap tmap) {
  using T = KindTraits<KIND>;
  extern __shared__ uint8_t smem_raw[];
  const uint32_t base_addr = smem_u32(smem_raw);
  const uint32_t pad = (128u - (base_addr & 127u)) & 127u;
  MeshSmem& sm = *reinterpret_cast<MeshSmem*>(smem_raw + pad);
  uint8_t* const mat = smem_raw + pad + sizeof(MeshSmem);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  uint32_t cur = p.use_queue ? 0u : blockIdx.x, end = 0, pending = 0;

  if (tid == 0) {
    mbar_init(&sm.bar, 1);
    sm.chunk_quads = 0;
    sm.task_next = 0;
    sm.any_solid = 0;
    fence_proxy_async_smem();
    if (p.use_queue && !T::kBrick) pending = atomicAdd(p.ticket, p.per_ticket);
  }
  for (int i = tid; i < 6 * 32; i += kThreads) (&sm.halo[0][0])[i] = 0;
  if (tid < 6) sm.rest_slices[tid] = 0;
  __syncthreads();

  uint32_t phase = 0;
  uint32_t qc = 0;  // quads staged in qbuf[warp] (warp-uniform)
  int bc = -1;         // brick maps: warp 0's ticket entries (see issue_chunk)
  uint32_t bmask = 0;
  for (;;) {
    if (warp == 0) issue_chunk<KIND>(sm, mat, p, &tmap, lane, cur, end, pending, bc, bmask);
    __syncthreads();
    const int c = sm.chunk;
    if (c < 0) break;
    // valid: 1 = mesh it; 0 = bad coordinate (flagged); 2 = no occupied brick
    const bool valid = sm.valid == 1;
    if constexpr (T::kBrick) {
      if (valid) {
        // 64 bricks x 64 pieces of 16 bytes; a warp covers 512 contiguous
        // bytes of one brick
#pragma unroll
        for (int k = 0; k < 4096 / kThreads; k++) {
          const int i = tid + kThreads * k, b = i >> 6, piece = i & 63;
          const uint32_t bp = sm.bptr[b];
          uint8_t* d = mat + b * kBrickSlot + 16 * piece;
          if (bp != MESO_EMPTY_BRICK)
            cp_async16(d, reinterpret_cast<const uint8_t*>(p.bmat) + (size_t)bp * 1024u + 16u * piece);
          else
            *reinterpret_cast<uint4*>(d) = make_uint4(0, 0, 0, 0);
        }
        cp_async_commit();
      }
    }
    if constexpr (T::kHalo) {
      if (valid) compute_halos<KIND>(sm, p, warp, lane);
    }
    if constexpr (T::kBrick) {
      if (valid) cp_async_wait_all();
    }
    const bool ok = mbar_wait_bounded(&sm.bar, phase, kWaitLimitNs);
    phase ^= 1u;
    if (__syncthreads_or(!ok)) {
      // the copy did not land within the limit: flag it, give it one more
      // bounded wait so nothing is in flight into shared memory, and leave
      if (tid == 0) {
        atomicOr(p.err, ERR_TIMEOUT);
        mbar_wait_bounded(&sm.bar, phase ^ 1u, kWaitLimitNs);
      }
      __syncthreads();
      return;
    }
    if (valid) {
      const uint8_t* mb = mat;
      // ---- pass 1: the warp pair of row group g builds slabs z0 .. z0+3
      // (z0 = 4g; lanes = x), warp w < 8 rows 0..15 and warp w + 8 rows
      // 16..31, 8 rows of the 4 slabs at a time, so the previous slab's
      // materials are still in registers for the -z equality.  Row words come
      // from ballots and are stored by lane 0; after a pair barrier each warp
      // makes the transposed copies (for the X faces) of two of the slabs.
      {
        const int g = warp & 7, half = warp >> 3;
        const int z0 = g * 4, ybeg = half * 16;
        uint32_t prev_m[4];  // row y0-1 of each slab
#pragma unroll
        for (int j = 0; j < 4; j++) prev_m[j] = half ? load_mat<KIND>(mb, lane, ybeg - 1, z0 + j) : 0u;
#pragma unroll 1
        for (int y0 = ybeg; y0 < ybeg + 16; y0 += 8) {
          uint32_t mp[8];  // rows y0 .. y0+7 of the slab below
#pragma unroll
          for (int k = 0; k < 8; k++) mp[k] = z0 > 0 ? load_mat<KIND>(mb, lane, y0 + k, z0 - 1) : 0u;
#pragma unroll
          for (int j = 0; j < 4; j++) {
            const int z = z0 + j, o = z * kS + y0;
            if (rows8_empty<KIND>(mb, y0, z, lane)) {
              if (lane < 8) {
                sm.occ[o + lane] = 0;
                sm.ex[o + lane] = 0;
                sm.ey[o + lane] = 0;
                sm.ez[o + lane] = 0;
              }
#pragma unroll
              for (int k = 0; k < 8; k++) mp[k] = 0;
              prev_m[j] = 0;
              continue;
            }
            uint32_t m[8];
#pragma unroll
            for (int k = 0; k < 8; k++) m[k] = load_mat<KIND>(mb, lane, y0 + k, z);
#pragma unroll
            for (int k = 0; k < 8; k++) {
              const uint32_t ml = __shfl_up_sync(kFull, m[k], 1);
              const uint32_t occw = __ballot_sync(kFull, m[k] != 0);
              const uint32_t exw = __ballot_sync(kFull, m[k] == ml);
              const uint32_t eyw = __ballot_sync(kFull, m[k] == (k ? m[k - 1] : prev_m[j]));
              const uint32_t ezw = __ballot_sync(kFull, m[k] == mp[k]);
              if (lane == 0) {
                sm.occ[o + k] = occw;
                sm.ex[o + k] = exw;
                sm.ey[o + k] = eyw;
                sm.ez[o + k] = ezw;
              }
            }
            prev_m[j] = m[7];
#pragma unroll
            for (int k = 0; k < 8; k++) mp[k] = m[k];
          }
        }
        // the pair's other warp builds the other half of these slabs' rows
        pair_sync(g);
#pragma unroll 1
        for (int j = 2 * half; j < 2 * half + 2; j++) {
          const int o = (z0 + j) * kS + lane;
          const uint32_t r_occ = sm.occ[o];
          uint32_t occT = 0, eyT = 0, ezT = 0;
          if (__any_sync(kFull, r_occ != 0)) {  // an empty slab needs no transposes
            occT = transpose32(r_occ, lane);
            eyT = transpose32(sm.ey[o], lane);
            ezT = transpose32(sm.ez[o], lane);
            if (lane == 0) sm.any_solid = 1;
          }
          sm.occt[o] = occT;
          sm.eyt[o] = eyT;
          sm.ezt[o] = ezT;
        }
      }
      __syncthreads();
      int32_t pf_a = -1, pf_b = 0, pf_c = 0;
      if (tid == 0) next_chunk<KIND>(p, cur, end, pending, pf_a, pf_b, pf_c);
      if (sm.any_solid) {
        // ---- pass 2: isolated faces (no same-material face neighbour in
        // the plane).  Quads never leave a component of same-material,
        // edge-adjacent faces, so these are 1x1 quads whatever the greedy
        // does elsewhere: they are peeled off into registers.  Warp w holds
        // rows v0 .. v0+3 (v0 = 4 (w mod 8)) of three directions (0-2 for
        // w < 8, 3-5 for the others; lane = slice), walking the rows in order
        // so the face words of the rows above and below are carried, not
        // recomputed.
        const int v0 = (warp & 7) * 4, dbase = (warp >> 3) * 3;
        uint32_t isow[kGroups];
        uint32_t lane_iso = 0;
        if (dbase) isolated_rows<3>(sm, v0, lane, isow, lane_iso);
        else isolated_rows<0>(sm, v0, lane, isow, lane_iso);
        const uint32_t total = __reduce_add_sync(kFull, lane_iso);
        unsigned long long run = 0;
        if (lane == 0 && total) run = atomicAdd(p.count, (unsigned long long)total);
        run = __shfl_sync(kFull, run, 0);
        uint32_t mine = total;
        const uint64_t chunk_bits = (uint64_t)((p.chunk_id_base + (uint32_t)c) & 0xFFFFFu) << 44;
        if (tid == 0) prefetch_chunk<KIND>(p, &tmap, pf_a, pf_b, pf_c);
        // the slices' rest flags are complete after this barrier; each warp
        // then emits its own isolated quads and pulls greedy tasks as soon as
        // it is done, so uneven emission work does not idle warps at a barrier
        __syncthreads();
        // ---- pass 3: isolated quads of this warp's words, the 4 rows of one
        // direction at a time (lane = slice).  A warp-balanced expansion over
        // all set bits of the 4 x 32 words: lane j of a round takes the
        // (32k+j)-th bit; its owning lane comes from a binary search over
        // the lanes' exclusive prefixes, the row from the owner's packed
        // running counts, the word from the warp's staging buffer (its
        // greedy staging area, empty at this point), the column from a
        // popcount-halving select.
        uint32_t* const stage = reinterpret_cast<uint32_t*>(sm.qbuf[warp]);  // [row q][lane]
#pragma unroll 1
        for (int dir = dbase; dir < dbase + 3; dir++) {
          // this direction's words are isow[0..3]; the rest shift down by 4
          const uint32_t w0 = isow[0], w1 = isow[1], w2 = isow[2], w3 = isow[3];
#pragma unroll
          for (int i = 0; i + 4 < kGroups; i++) isow[i] = isow[i + 4];
          const uint32_t c1 = __popc(w0), c2 = c1 + __popc(w1), c3 = c2 + __popc(w2);
          const uint32_t n = c3 + __popc(w3);
          uint32_t incl = n;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(kFull, incl, o);
            if (lane >= o) incl += y;
          }
          const uint32_t G = __shfl_sync(kFull, incl, 31);
          if (G == 0) continue;
          const uint32_t ex = incl - n;
          // running counts before rows 1, 2, 3 in bytes 1..3 (byte 0: 0)
          const uint32_t packed = c1 << 8 | c2 << 16 | c3 << 24;
          stage[lane] = w0;
          stage[32 + lane] = w1;
          stage[64 + lane] = w2;
          stage[96 + lane] = w3;
          __syncwarp();
          // run: this direction's first output index (the warp reserved all
          // three directions' isolated quads at once, after pass 2)
          const bool all_fit = run + G <= p.cap;
          uint2* const dst = reinterpret_cast<uint2*>(p.quads) + run;
          // bit offsets of slice, column and row in the linear voxel index
          const int sh_s = dir < 2 ? 0 : (dir < 4 ? 5 : 10);
          const int sh_u = dir < 2 ? 5 : 0;
          const int sh_v = dir < 4 ? 10 : 5;
          const uint32_t hi_bits = (uint32_t)(chunk_bits >> 32) | (uint32_t)dir << 9;
          auto emit = [&](uint32_t j, int l) {
            const uint32_t r = j - __shfl_sync(kFull, ex, l);
            const uint32_t pk = __shfl_sync(kFull, packed, l);
            if (j < G) {
              const uint32_t q = (uint32_t)(r >= ((pk >> 8) & 0xFFu)) + (uint32_t)(r >= ((pk >> 16) & 0xFFu)) +
                                 (uint32_t)(r >= (pk >> 24));
              const uint32_t rb = (pk >> (8 * q)) & 0xFFu;
              const uint32_t u = select_bit(stage[32 * q + l], r - rb);
              const uint32_t lin = (uint32_t)l << sh_s | u << sh_u | ((uint32_t)v0 + q) << sh_v;
              const uint32_t mat = load_mat_lin<KIND>(mb, lin);
              if (all_fit || run + j < p.cap) dst[j] = make_uint2(lin << 26 | mat, hi_bits | lin >> 6);
            }
          };
          // two rounds (64 bits) per pass, so their shuffle chains interleave
          for (uint32_t k2 = 0; k2 < G; k2 += 64) {
            const uint32_t ja = k2 + (uint32_t)lane, jb = ja + 32u;
            int la = 0, lb = 0;
#pragma unroll
            for (int step = 16; step >= 1; step >>= 1) {
              const uint32_t oa = __shfl_sync(kFull, ex, la + step);
              const uint32_t ob = __shfl_sync(kFull, ex, lb + step);
              if (oa <= ja) la += step;
              if (ob <= jb) lb += step;
            }
            emit(ja, la);
            if (k2 + 32u < G) emit(jb, lb);
          }
          run += G;
          __syncwarp();  // the stage is rewritten by the next direction
        }
        // ---- pass 4: greedy on the remaining faces, one warp per slice.
        // Lane r holds row r of the slice in registers: its faces (isolated
        // ones removed again), their equality with the -u and -v neighbours,
        // and the bits consumed so far.  Rows are scanned in order; in a row
        // every maximal run of unconsumed same-material faces is one quad
        // (Lysenko's left-to-right scan gives exactly these runs); a quad's
        // height is one ballot over the rows below, and the quads of one row
        // never interact because their columns are disjoint.
        uint32_t rs[6], pre[6];
        uint32_t n_tasks = 0;
#pragma unroll
        for (int d = 0; d < 6; d++) {
          rs[d] = sm.rest_slices[d];
          pre[d] = n_tasks;
          n_tasks += __popc(rs[d]);
        }
        uint64_t* qb = sm.qbuf[warp];
        for (;;) {
          uint32_t t = 0;
          if (lane == 0) t = atomicAdd(&sm.task_next, 1u);
          t = __shfl_sync(kFull, t, 0);
          if (t >= n_tasks) break;
          int dir = 0;
          uint32_t before = 0, smask = rs[0];
#pragma unroll
          for (int d = 1; d < 6; d++) {
            if (t >= pre[d]) {
              dir = d;
              before = pre[d];
              smask = rs[d];
            }
          }
          const int sl = (int)select_bit(smask, t - before);
          const int orow = word_off(dir, sl, lane);
          const uint32_t F0 = face_col(sm, dir, sl, lane);
          const uint32_t Er = e_arr(sm, dir)[orow];
          const uint32_t Vr = v_arr(sm, dir)[orow];
          uint32_t fu = __shfl_up_sync(kFull, F0, 1), fd = __shfl_down_sync(kFull, F0, 1);
          uint32_t vd = __shfl_down_sync(kFull, Vr, 1);
          if (lane == 0) fu = 0;
          if (lane == 31) fd = vd = 0;
          // the faces pass 2 left: not isolated and not in a domino
          const uint32_t hl = F0 & Er & (F0 << 1), hh = hl | (hl >> 1);
          const uint32_t ul = F0 & Vr & fu, dl = F0 & vd & fd, vl = ul | dl;
          const uint32_t hd = hl & ~(hl << 1) & ~(hl >> 1) & ~vl & ~(vl << 1);
          uint32_t hn = __shfl_down_sync(kFull, hh, 1), dn = __shfl_down_sync(kFull, dl, 1);
          if (lane == 31) hn = dn = 0;
          const uint32_t vdt = dl & ~hh & ~ul & ~hn & ~dn;
          uint32_t vdb = __shfl_up_sync(kFull, vdt, 1);
          if (lane == 0) vdb = 0;
          const uint32_t Fr = F0 & (hh | vl) & ~(hd | (hd >> 1) | vdt | vdb);
          {
            // two-face components first: a 2x1 or 1x2 quad whatever the
            // scan order (origins hd >> 1: 2 wide, vdt: 2 high; lane = row)
            uint32_t ho = hd >> 1, vo = vdt;
            while (__any_sync(kFull, (ho | vo) != 0u)) {
              const bool horiz = ho != 0u;
              const uint32_t act = __ballot_sync(kFull, (ho | vo) != 0u);
              const uint32_t n = __popc(act);
              if (qc + n > (uint32_t)kQBuf) {
                flush_warp(sm, warp, p, lane, qc);
                qc = 0;
              }
              if (ho | vo) {
                uint32_t u;
                if (horiz) {
                  u = __ffs(ho) - 1;
                  ho &= ho - 1u;
                } else {
                  u = __ffs(vo) - 1;
                  vo &= vo - 1u;
                }
                int x, y, z;
                face_xyz(dir, sl, (int)u, lane, x, y, z);
                const uint32_t mat = load_mat<KIND>(mb, x, y, z);
                qb[qc + __popc(act & lanemask_lt())] =
                    chunk_bits | (uint64_t)dir << 41 | (uint64_t)z << 36 | (uint64_t)y << 31 | (uint64_t)x << 26 |
                    (uint64_t)(horiz ? 1u : 0u) << 21 | (uint64_t)(horiz ? 0u : 1u) << 16 | (uint64_t)mat;
              }
              qc += n;
              mine += n;
            }
          }
          uint32_t rows = __ballot_sync(kFull, Fr != 0);
          const uint64_t dir_bits = chunk_bits | (uint64_t)dir << 41;
          uint32_t cons = 0;
          while (rows) {
            const int v = __ffs(rows) - 1;
            rows &= rows - 1;
            const uint32_t cur = Fr & ~cons;
            const uint32_t word = __shfl_sync(kFull, cur, v);
            if (!word) continue;
            const uint32_t e = __shfl_sync(kFull, Er, v);
            const uint32_t link = word & e & (word << 1);
            const uint32_t starts = word & ~link;
            const uint32_t cnt = __popc(starts);
            if (qc + cnt > (uint32_t)kQBuf) {
              flush_warp(sm, warp, p, lane, qc);
              qc = 0;
            }
            const uint32_t q0 = qc;
            // every start lane grows its quad; row r's words come from lane r
            const bool is_start = (starts >> lane) & 1u;
            const int w = __ffs(~__funnelshift_rc(link, 0u, (uint32_t)lane + 1u));
            const uint32_t mask = is_start ? ((2u << (w - 1)) - 1u) << lane : 0u;
            const uint32_t grow = Fr & Vr;  // faces that continue the row above in material
            bool active = is_start;
            int h = 1;
            // two rows per step: row r+1's word is fetched with row r's (a
            // row's consumed bits change only when its own turn comes)
            for (int r = v + 1; r < 32; r += 2) {
              const uint32_t gr = grow & ~cons;
              const uint32_t g0 = __shfl_sync(kFull, gr, r);
              const uint32_t g1 = __shfl_sync(kFull, gr, r + 1 < 32 ? r + 1 : 31);
              const bool c0 = active && (g0 & mask) == mask;
              const bool c1 = c0 && r + 1 < 32 && (g1 & mask) == mask;
              const uint32_t t0 = __reduce_or_sync(kFull, c0 ? mask : 0u);
              const uint32_t t1 = __reduce_or_sync(kFull, c1 ? mask : 0u);
              if (lane == r) cons |= t0;
              if (lane == r + 1) cons |= t1;
              h += (c0 ? 1 : 0) + (c1 ? 1 : 0);
              active = c1;
              if (!__any_sync(kFull, active)) break;
            }
            if (is_start) {
              int x, y, z;
              face_xyz(dir, sl, lane, v, x, y, z);
              const uint32_t mat = load_mat<KIND>(mb, x, y, z);
              qb[q0 + __popc(starts & lanemask_lt())] = dir_bits | (uint64_t)z << 36 | (uint64_t)y << 31 |
                                                         (uint64_t)x << 26 | (uint64_t)(w - 1) << 21 |
                                                         (uint64_t)(h - 1) << 16 | (uint64_t)mat;
            }
            qc = q0 + cnt;
            mine += cnt;
          }
        }
        if (p.chunk_counts && lane == 0 && mine) atomicAdd(&sm.chunk_quads, mine);
        if (qc) {  // the staging area doubles as pass 3's word buffer
          flush_warp(sm, warp, p, lane, qc);
          qc = 0;
        }
      }
    }
    __syncthreads();
    if (tid == 0) {
      if (p.chunk_counts) p.chunk_counts[c] = valid ? sm.chunk_quads : 0u;
      sm.chunk_quads = 0;
      sm.task_next = 0;
      sm.any_solid = 0;
    }
    if (tid < 6) sm.rest_slices[tid] = 0;
  }
  flush_warp(sm, warp, p, lane, qc);
}

// --------------------------------------------------------------- host side

PFN_cuTensorMapEncodeTiled_v12000 get_encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  });
  return fn;
}

meso_status make_grid_map(const meso_mesh_source* src, int elem, CUtensorMap* map) {
  auto enc = get_encode_fn();
  if (!enc) return fail(MESO_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  cuuint64_t dims[3] = {(cuuint64_t)src->nx, (cuuint64_t)src->ny, (cuuint64_t)src->nz};
  cuuint64_t strides[2] = {(cuuint64_t)src->nx * elem, (cuuint64_t)src->nx * src->ny * elem};
  cuuint32_t box[3] = {32, 32, 32};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = enc(map, elem == 2 ? CU_TENSOR_MAP_DATA_TYPE_UINT16 : CU_TENSOR_MAP_DATA_TYPE_UINT8, 3,
                   const_cast<void*>(src->d_data), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                   CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(MESO_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
  return MESO_OK;
}

template <int KIND>
meso_status launch_kind(meso_ctx* ctx, const MeshParams& base, const CUtensorMap& tmap, uint32_t n_chunks,
                        cudaStream_t st, bool per_launch) {
  const size_t smem = sizeof(MeshSmem) + KindTraits<KIND>::kMatBytes + 128;
  static bool attr_set[64] = {false};
  if (!attr_set[ctx->device & 63]) {
    MESO_CUDA_TRY(cudaFuncSetAttribute(mesh_kernel<KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    MESO_CUDA_TRY(cudaFuncSetAttribute(mesh_kernel<KIND>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                       (int)cudaSharedmemCarveoutMaxShared));
    attr_set[ctx->device & 63] = true;
  }
  constexpr bool kCoords3 = KindTraits<KIND>::kGrid || KindTraits<KIND>::kBrick;
  if (per_launch) {
    for (uint32_t i = 0; i < n_chunks; i++) {
      MeshParams p = base;
      p.n_chunks = 1;
      p.chunk_id_base = base.chunk_id_base + i;
      p.use_queue = 0;
      if (kCoords3) p.coords = base.coords + 3 * (size_t)i;
      else if (base.coords) p.coords = base.coords + i;
      else p.data = base.data + (size_t)i * 32768u * KindTraits<KIND>::kElem;
      if (p.chunk_counts) p.chunk_counts = base.chunk_counts + i;
      mesh_kernel<KIND><<<1, kThreads, smem, st>>>(p, tmap);
      ctx->launches.fetch_add(1);
    }
    MESO_CUDA_TRY(cudaGetLastError());
    return MESO_OK;
  }
  MeshParams p = base;
  p.use_queue = 1;
  // CTAs per SM: the tuned value, at most (and by default) what fits the SM
  constexpr uint32_t kMaxCtas = KindTraits<KIND>::kCtasPerSm;
  const uint32_t tuned = ctx->tuning.mesh_ctas_per_sm;
  uint32_t grid = ctx->sm_count * (tuned && tuned < kMaxCtas ? tuned : kMaxCtas);
  if constexpr (KindTraits<KIND>::kBrick) {
    // tickets of up to 8 list entries (tested together against the cell
    // map) once every CTA gets several: on all 32,768 chunks of a 1024^3
    // terrain (80 % air) tickets of 4 or 8 measured 0.84 ms, 16 0.87, 32 0.92
    // (the last tickets leave CTAs with several heavy chunks each).  7919 and
    // 104729 are primes, and no list of at most 2^20 entries is a multiple of
    // both, so t -> (t * perm_mul) mod n is a bijection
    const uint32_t b = n_chunks / grid;
    p.per_ticket = b < 1 ? 1 : (b > 8 ? 8 : b);
    p.perm_mul = n_chunks % 7919u ? 7919u : 104729u;
  }
  const uint32_t per = p.per_ticket ? p.per_ticket : 1;
  const uint32_t need = (n_chunks + per - 1) / per;
  if (grid > need) grid = need;
  if (grid == 0) grid = 1;
  MESO_CUDA_TRY(cudaMemsetAsync(p.ticket, 0, sizeof(uint32_t), st));
  mesh_kernel<KIND><<<grid, kThreads, smem, st>>>(p, tmap);
  ctx->launches.fetch_add(1);
  MESO_CUDA_TRY(cudaGetLastError());
  return MESO_OK;
}

}  // namespace

meso_status launch_mesh(meso_ctx* ctx, const meso_mesh_source* src, const int32_t* d_coords, uint32_t n_chunks,
                        const meso_mesh_output* out, cudaStream_t st, bool per_launch, uint32_t chunk_id_base,
                        bool accumulate) {
  if (!src || !out || !out->d_quad_count) return fail(MESO_ERR_INVALID_ARG, "mesh: null source/output");
  if ((uint64_t)chunk_id_base + n_chunks > MESO_MAX_CHUNKS_PER_CALL)
    return fail(MESO_ERR_INVALID_ARG, "mesh: more than 2^20 chunks");
  if (out->capacity && !out->d_quads) return fail(MESO_ERR_INVALID_ARG, "mesh: capacity without buffer");
  MeshParams p;
  memset(&p, 0, sizeof(p));
  p.coords = d_coords;
  p.n_chunks = n_chunks;
  p.quads = out->d_quads;
  p.cap = out->capacity;
  p.count = reinterpret_cast<unsigned long long*>(out->d_quad_count);
  p.chunk_counts = out->d_chunk_quad_counts;
  p.ticket = ctx->d_tickets + (ctx->next_ticket.fetch_add(1) % meso_ctx::kTicketRing);
  p.err = ctx->d_scratch + 1;
  p.per_ticket = ctx->tuning.mesh_chunks_per_ticket ? ctx->tuning.mesh_chunks_per_ticket : 1;
  p.chunk_id_base = chunk_id_base;
  CUtensorMap tmap;
  memset(&tmap, 0, sizeof(tmap));
  const int kind = src->kind;
  if (kind == MESO_SRC_BRICKMAP) {
    const meso_scene* s = src->scene;
    if (!s) return fail(MESO_ERR_INVALID_ARG, "mesh: brick-map source without scene");
    if (s->nx % 32 || s->ny % 32 || s->nz % 32) return fail(MESO_ERR_INVALID_ARG, "mesh: scene dims not multiples of 32");
    if (!d_coords && n_chunks) return fail(MESO_ERR_INVALID_ARG, "mesh: brick-map source needs chunk coordinates");
    p.bptr = s->d_ptr;
    p.bocc = s->d_occ;
    p.bmat = s->d_mat;
    p.bcell = s->d_macro;
    p.bx = s->bx;
    p.by = s->by;
    p.bz = s->bz;
  } else {
    if (!src->d_data && n_chunks) return fail(MESO_ERR_INVALID_ARG, "mesh: null data");
    p.data = static_cast<const uint8_t*>(src->d_data);
    p.nx = src->nx;
    p.ny = src->ny;
    p.nz = src->nz;
    if (kind == MESO_SRC_GRID_U8 || kind == MESO_SRC_GRID_U16) {
      if (src->nx <= 0 || src->ny <= 0 || src->nz <= 0 || src->nx % 32 || src->ny % 32 || src->nz % 32)
        return fail(MESO_ERR_INVALID_ARG, "mesh: grid dims must be positive multiples of 32");
      if (!d_coords && n_chunks) return fail(MESO_ERR_INVALID_ARG, "mesh: grid source needs chunk coordinates");
      if ((reinterpret_cast<uintptr_t>(src->d_data) & 15u) != 0)
        return fail(MESO_ERR_INVALID_ARG, "mesh: grid base must be 16-byte aligned");
      MESO_TRY(make_grid_map(src, kind == MESO_SRC_GRID_U16 ? 2 : 1, &tmap));
    } else if (kind == MESO_SRC_CHUNKS_U16 || kind == MESO_SRC_CHUNKS_U8) {
      if ((reinterpret_cast<uintptr_t>(src->d_data) & 15u) != 0)
        return fail(MESO_ERR_INVALID_ARG, "mesh: chunk array must be 16-byte aligned");
      if (d_coords && src->nx <= 0)
        return fail(MESO_ERR_INVALID_ARG, "mesh: an index list needs nx = number of chunks in the array");
    } else {
      return fail(MESO_ERR_INVALID_ARG, "mesh: unknown source kind");
    }
  }
  if (!accumulate) MESO_CUDA_TRY(cudaMemsetAsync(out->d_quad_count, 0, sizeof(uint64_t), st));
  if (n_chunks == 0) return MESO_OK;
  switch (kind) {
    case MESO_SRC_CHUNKS_U16: return launch_kind<MESO_SRC_CHUNKS_U16>(ctx, p, tmap, n_chunks, st, per_launch);
    case MESO_SRC_CHUNKS_U8: return launch_kind<MESO_SRC_CHUNKS_U8>(ctx, p, tmap, n_chunks, st, per_launch);
    case MESO_SRC_GRID_U8: return launch_kind<MESO_SRC_GRID_U8>(ctx, p, tmap, n_chunks, st, per_launch);
    case MESO_SRC_GRID_U16: return launch_kind<MESO_SRC_GRID_U16>(ctx, p, tmap, n_chunks, st, per_launch);
    default: return launch_kind<MESO_SRC_BRICKMAP>(ctx, p, tmap, n_chunks, st, per_launch);
  }
}


}  // namespace meso
