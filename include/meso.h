/*
 * meso.h -- C ABI of mesoengine_gb300: GB300-native (sm_103a) voxel-chunk
 * greedy meshing and two-level brick-map raymarching.
 *
 * The reference MesoEngine exposes these paths as in-process C++ classes,
 * not as an FFI; each entry point below names the reference call it stands
 * in for (path:line inside the MesoEngine tree).  Conventions kept from the
 * reference:
 *   - linear index x + y*Rx + z*Rx*Ry, x fastest
 *     (Runtimes/Helper/VoxelMathHelper.h:73-76);
 *   - chunk -> 8^3 brick -> voxel, one brick pointer per brick
 *     (Runtimes/Voxel/VoxelStructure.h:14-15, Runtimes/Voxel/Block/Block.h:18);
 *   - all-ones pointer = empty brick, like the reference's INT_MAX "invalid"
 *     sentinels (Runtimes/Voxel/Block/Block.h:16-18, Runtimes/Voxel/Chunk/Chunk.h:29);
 *   - camera given as an integer chunk plus a fractional offset, z-up
 *     (Runtimes/Instance/VoxelCamera.cpp:42-59, Runtimes/Instance/VoxelCamera.h:23).
 *
 * Errors: every call returns meso_status; no exception crosses the ABI.
 * meso_last_error_string() gives a message for the calling thread.
 * Streams are passed as void* (a cudaStream_t; NULL = the context's stream).
 * Device pointers are marked d_, host pointers h_.
 */
#ifndef MESO_H
#define MESO_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MESO_CHUNK_EDGE 32u
#define MESO_BRICK_EDGE 8u
#define MESO_EMPTY_BRICK 0xFFFFFFFFu
#define MESO_MAX_CHUNKS_PER_CALL (1u << 20)

typedef enum meso_status {
  MESO_OK = 0,
  MESO_ERR_INVALID_ARG = 1,
  MESO_ERR_OOM = 2,
  MESO_ERR_OVER_BUDGET = 3,
  MESO_ERR_OVERFLOW = 4, /* output capacity too small; the count holds the need */
  MESO_ERR_TIMEOUT = 5,  /* a bounded device wait gave up */
  MESO_ERR_CUDA = 6,
  MESO_ERR_NOT_READY = 7,
  MESO_ERR_SHUTDOWN = 8
} meso_status;

/* ------------------------------------------------------------------ context */

/* Replaces FVoxelSceneConfig (Runtimes/Voxel/VoxelSceneConfig.h:20-49): the
 * chunk/brick resolution plus the batching knobs that take the place of
 * ChunkTaskPerCore / MaxUnsyncedLoadChunkCount. Zero fields take defaults. */
typedef struct meso_config {
  uint32_t chunk_edge;            /* must be 32 (or 0) */
  uint32_t brick_edge;            /* must be 8 (or 0) */
  int32_t device;                 /* CUDA device ordinal */
  uint32_t mesh_ctas_per_sm;      /* persistent mesher CTAs (16 warps each) per SM, 1..2
                                     (0 = tuned/default 2) */
  uint32_t mesh_chunks_per_ticket;/* chunks taken per queue ticket (0 = tuned/default 1); brick-map
                                     sources size their tickets themselves (up to 8 chunks, tested
                                     together against the scene's cell map) */
  uint32_t ray_tile_w, ray_tile_h;/* threads of one ray CTA tile (0 = tuned/default 8x4 per warp) */
  uint32_t ray_warps_per_cta;     /* 1..4, 0 = tuned/default */
  uint64_t hbm_budget_bytes;      /* admission budget for resident scenes + requests (0 = 90% of free) */
  const char* tuning_path;        /* optional tuning JSON written by meso_autotune */
} meso_config;

typedef struct meso_ctx meso_ctx;
typedef struct meso_scene meso_scene;

/* Stands in for FChunkManage::Initialize (Runtimes/Voxel/Chunk/ChunkManager.h:90-102):
 * binds a device instead of spawning a host ThreadPool (Runtimes/Thread/ThreadPool.h:25-43).
 * Per-call temporaries come from the device's default stream-ordered memory
 * pool; this raises that pool's release threshold (a per-process attribute)
 * to at least 1 GiB so freed blocks are reused rather than remapped. */
meso_status meso_ctx_create(const meso_config* cfg, meso_ctx** out);
void meso_ctx_destroy(meso_ctx* ctx);
const char* meso_last_error_string(void);
const char* meso_status_string(meso_status s);
meso_status meso_sync(meso_ctx* ctx, void* stream);
/* The context's effective configuration: defaults filled in, tuning file
 * and autotuning applied (tuning_path is returned as NULL). */
meso_status meso_ctx_get_config(const meso_ctx* ctx, meso_config* out);
/* Number of mesher/raymarch/scene kernels this context has launched. */
uint64_t meso_kernel_launches(const meso_ctx* ctx);
int meso_sm_count(const meso_ctx* ctx);
/* Diagnostic of the failure path (no counterpart in the reference): runs a
 * kernel whose bounded device wait cannot succeed (an mbarrier nothing
 * arrives on, waited for with the helper that guards every TMA copy of the
 * mesher).  The wait gives up after limit_us (1 .. 1,000,000), the kernel
 * flags the timeout and exits, and the call returns MESO_ERR_TIMEOUT; the
 * context stays usable. */
meso_status meso_selftest_bounded_wait(meso_ctx* ctx, uint32_t limit_us);
/* Measurement helper (no counterpart in the reference): the L2 read
 * bandwidth, the denominator for work whose fetches hit in L2 (the
 * raymarch's).  A device buffer of `bytes` (16 KiB .. 64 MiB, a multiple of
 * 16, so it stays in L2) is read once untimed and then `passes` times
 * (1..1000) with 16-byte loads that bypass L1; *gb_s = bytes * passes / time. */
meso_status meso_measure_l2_read(meso_ctx* ctx, uint64_t bytes, uint32_t passes, double* gb_s);

/* Device memory, streams and events for callers without another CUDA host
 * library (tests, the Python binding). */
meso_status meso_dev_alloc(meso_ctx* ctx, size_t bytes, void** d_ptr);
meso_status meso_dev_free(meso_ctx* ctx, void* d_ptr);
meso_status meso_host_alloc_pinned(meso_ctx* ctx, size_t bytes, void** h_ptr);
meso_status meso_host_free_pinned(meso_ctx* ctx, void* h_ptr);
meso_status meso_memcpy_h2d(meso_ctx* ctx, void* d_dst, const void* h_src, size_t bytes, void* stream);
meso_status meso_memcpy_d2h(meso_ctx* ctx, void* h_dst, const void* d_src, size_t bytes, void* stream);
meso_status meso_memset(meso_ctx* ctx, void* d_dst, int value, size_t bytes, void* stream);
meso_status meso_stream_create(meso_ctx* ctx, void** stream);
meso_status meso_stream_destroy(meso_ctx* ctx, void* stream);
meso_status meso_event_create(meso_ctx* ctx, void** ev);
meso_status meso_event_destroy(meso_ctx* ctx, void* ev);
meso_status meso_event_record(meso_ctx* ctx, void* ev, void* stream);
meso_status meso_event_elapsed_ms(meso_ctx* ctx, void* ev_start, void* ev_end, float* ms);

/* ----------------------------------------------------------------- scenes */

/* Terrain generator (replaces FGeneratorHelper::GenerateSphere / TestGenerator,
 * Runtimes/Helper/GeneratorHelper.h:19-150, whose sin-hash cannot be
 * reproduced bit for bit across host and device).  Solid iff
 * z < H0 + amp*fbm(x,y) and the 3-D value noise (cave_period) does not
 * exceed cave_threshold; material 1 + ((floor(h) - z) / 4 mod 64). */
typedef struct meso_terrain {
  int32_t nx, ny, nz; /* voxels, multiples of 32 */
  uint32_t seed;
  uint32_t height_period;
  int32_t height_octaves;
  float height_base;
  float height_amp;
  uint32_t cave_period;
  float cave_threshold;
} meso_terrain;

typedef struct meso_scene_info {
  int32_t nx, ny, nz;
  uint64_t n_bricks;        /* live bricks */
  uint64_t brick_capacity;  /* pool slots */
  uint64_t device_bytes;    /* pointer grid + pools */
  const uint32_t* d_ptr;    /* (nx/8)(ny/8)(nz/8) brick pointers */
  const uint64_t* d_occ;    /* 8 words per brick slot, word z, bit x+8y */
  const uint16_t* d_mat;    /* 512 materials per brick slot, x+8y+64z */
} meso_scene_info;

/* Builds a brick-map scene on the device.  spare_bricks extra pool slots are
 * reserved for later edits.  Stands in for the generator threads of
 * FChunkManage::MultiThreadGeneratorBatched (Runtimes/Voxel/Chunk/ChunkManager.h:183-210)
 * and the pool writes of FChunkPool::PushChunk (Runtimes/Voxel/Chunk/ChunkPool.h:623-628). */
meso_status meso_scene_create_terrain(meso_ctx* ctx, const meso_terrain* t, uint64_t spare_bricks,
                                      meso_scene** out);
/* Uploads a dense uint16 grid (x fastest, dims multiples of 32) and builds
 * its brick map on the device. */
meso_status meso_scene_create_dense(meso_ctx* ctx, const uint16_t* h_grid, int32_t nx, int32_t ny,
                                    int32_t nz, uint64_t spare_bricks, meso_scene** out);
/* Builds the brick map of a dense grid already in device memory: kind
 * MESO_SRC_GRID_U8 (uint8 materials, widened to uint16) or MESO_SRC_GRID_U16;
 * x fastest, dims multiples of 32.  Lets a grid made on the device (e.g. by
 * meso_generate_dense_u8) be raymarched without a host round trip; the
 * reference's counterpart is the same pool write as for the terrain
 * (Runtimes/Voxel/Chunk/ChunkPool.h:623-628).  d_grid is only read. */
meso_status meso_scene_create_grid(meso_ctx* ctx, int32_t kind, const void* d_grid, int32_t nx, int32_t ny,
                                   int32_t nz, uint64_t spare_bricks, meso_scene** out);
/* Solid voxels of a scene (set occupancy bits of its linked bricks); for
 * reporting occupancy (no counterpart in the reference).  Waits for the
 * context's stream. */
meso_status meso_scene_count_solid(meso_ctx* ctx, const meso_scene* scene, uint64_t* n_solid);
meso_status meso_scene_destroy(meso_ctx* ctx, meso_scene* scene);
meso_status meso_scene_get_info(meso_ctx* ctx, const meso_scene* scene, meso_scene_info* info);
/* Copies the scene to the host: ptr has (nx/8)(ny/8)(nz/8) entries; occ and
 * mat receive brick_capacity slots (either may be NULL). */
meso_status meso_scene_download(meso_ctx* ctx, const meso_scene* scene, uint32_t* h_ptr, uint64_t* h_occ,
                                uint16_t* h_mat);

/* Dense generators for the meshing workloads (seeded, bit-identical to the
 * definitions in the documentation).  d_out is device memory. */
meso_status meso_generate_dense_u8(meso_ctx* ctx, int32_t nx, int32_t ny, int32_t nz, uint32_t seed,
                                   uint8_t* d_out, void* stream);
meso_status meso_generate_chunks_u16(meso_ctx* ctx, uint32_t n_chunks, uint32_t seed0, uint16_t* d_out,
                                     uint32_t* d_solid_count, void* stream);

/* ---------------------------------------------------------------- meshing */

/* Packed quad (uint64), most significant field first:
 *   [63:44] chunk index within the call   [43:41] dir 0 +X,1 -X,2 +Y,3 -Y,4 +Z,5 -Z
 *   [40:36] z  [35:31] y  [30:26] x  (chunk-local origin voxel)
 *   [25:21] w-1 along u   [20:16] h-1 along v   [15:0] material
 * Plane axes: X faces u=y,v=z; Y faces u=x,v=z; Z faces u=x,v=y.
 * Numeric order of the uint64 values is the canonical (chunk, dir, z, y, x)
 * order.  This replaces the reference's one-instance-per-visible-block
 * FGPUBlock stream (Runtimes/Voxel/Block/Block.h:21-65). */

typedef enum meso_source_kind {
  MESO_SRC_GRID_U8 = 0,    /* dense uint8 grid; faces see neighbours across chunks */
  MESO_SRC_CHUNKS_U16 = 1, /* array of standalone 32^3 uint16 chunks; outside = empty */
  MESO_SRC_BRICKMAP = 2,   /* brick-map scene; faces see neighbours across chunks */
  MESO_SRC_GRID_U16 = 3,   /* dense uint16 grid */
  MESO_SRC_CHUNKS_U8 = 4   /* array of standalone 32^3 uint8 chunks */
} meso_source_kind;

typedef struct meso_mesh_source {
  int32_t kind;             /* meso_source_kind */
  const void* d_data;       /* grid or chunk array (device); unused for bricks */
  int32_t nx, ny, nz;       /* grid dims (grid kinds), multiples of 32; chunk-array kinds:
                               nx = chunks in the array (needed with an index list) */
  const meso_scene* scene;  /* brick-map kind */
} meso_mesh_source;

typedef struct meso_mesh_output {
  uint64_t* d_quads;            /* capacity entries */
  uint64_t capacity;
  uint64_t* d_quad_count;       /* total quads produced (may exceed capacity) */
  uint32_t* d_chunk_quad_counts;/* optional, one per chunk */
} meso_mesh_output;

/* Meshes n_chunks chunks in ONE persistent launch fed by a device work queue.
 * d_chunk_coords: n_chunks int32 triples (grid/brick kinds) or n_chunks int32
 * chunk indices (chunk-array kinds; NULL = 0..n-1).  Replaces the host loop
 * FChunkManage::UpdateLoadingQueue -> MultiThreadGeneratorBatched ->
 * FChunkPool::PushToBlockPool (Runtimes/Voxel/Chunk/ChunkManager.h:211-400,
 * :183-210; Runtimes/Voxel/Chunk/ChunkPool.h:381-445).  Asynchronous on
 * stream; MESO_ERR_OVERFLOW is reported by meso_mesh_check. */
meso_status meso_mesh_chunks(meso_ctx* ctx, const meso_mesh_source* src, const int32_t* d_chunk_coords,
                             uint32_t n_chunks, const meso_mesh_output* out, void* stream);
/* The plain form: one kernel launch per chunk (the baseline the batched form
 * is measured against). */
meso_status meso_mesh_chunks_per_launch(meso_ctx* ctx, const meso_mesh_source* src,
                                        const int32_t* d_chunk_coords, uint32_t n_chunks,
                                        const meso_mesh_output* out, void* stream);
/* Synchronises stream, reads the quad count (always written to *h_count)
 * and the device error flag: MESO_ERR_INVALID_ARG when a chunk coordinate or
 * index was outside the source (that chunk yields no quads and count 0; the
 * other chunks' quads are in the buffer), MESO_ERR_OVERFLOW when the count
 * exceeds the capacity. */
meso_status meso_mesh_check(meso_ctx* ctx, const meso_mesh_output* out, void* stream, uint64_t* h_count);
/* Host-buffer form for callers that hold no device memory: copies the
 * chunk array (kind CHUNKS_U16/U8; nx chunks, or n_chunks when nx is 0) or
 * grid to the device, meshes, and returns the quads.  A contiguous chunk
 * array of more than 1024 chunks goes up in slices of 1024, each meshed
 * while the next one is copied; if h_quads is page-locked host memory the
 * kernel writes the quads into it directly, else they are copied back.
 * Quads carry the chunks' indices in the whole array.  *h_count receives the
 * number of quads (MESO_ERR_OVERFLOW if it exceeds capacity). */
meso_status meso_mesh_host(meso_ctx* ctx, int32_t kind, const void* h_data, int32_t nx, int32_t ny,
                           int32_t nz, const int32_t* h_chunk_coords, uint32_t n_chunks, uint64_t* h_quads,
                           uint64_t capacity, uint64_t* h_count);

/* -------------------------------------------------------------- raymarching */

/* Camera: FGPUUniformCamera (Runtimes/Shader/GPUStructures.h:36-56) recast
 * for ray generation.  Pixel ray: s_x = ((2px+1)/W - 1) tan_half_fov_y W/H,
 * s_y = (1 - (2py+1)/H) tan_half_fov_y, d = normalize(forward + s_x right + s_y up). */
typedef struct meso_camera {
  int32_t origin_chunk[3];
  float origin_frac[3];
  float forward[3];
  float right[3];
  float up[3];
  float tan_half_fov_y;
  uint32_t width, height;
} meso_camera;

/* Hit record (24 bytes). */
typedef struct meso_hit {
  uint64_t voxel;        /* x + y*nx + z*nx*ny; UINT64_MAX on a miss */
  float t;               /* distance to the entry of the hit voxel; +inf on a miss */
  uint16_t material;
  uint8_t face;          /* entered face normal 0 +X,1 -X,2 +Y,3 -Y,4 +Z,5 -Z; 6 none */
  uint8_t shadow;        /* 1 occluded, 0 lit, 255 not traced */
  uint32_t steps;        /* fine | coarse << 16 */
  uint32_t shadow_steps; /* fine | coarse << 16 */
} meso_hit;

#define MESO_RAY_SHADOW 1u

/* Marches every pixel of n_views cameras in ONE launch; view v reads scene
 * scenes[v] and writes its width*height hits after those of views 0..v-1.
 * Replaces the imposter draw (Samples/SimpleVoxel.cpp:374-393, vertex shader
 * :146-192).  light: normalised direction towards the light (MESO_RAY_SHADOW).
 * The walk is the two-level DDA (a coarse step per empty brick, a fine step
 * per voxel of an occupied brick); empty cells of 4^3, 16^3 and 64^3 bricks
 * are crossed in one jump whose result, step counts included, is that of the
 * brick-by-brick walk. */
meso_status meso_raymarch(meso_ctx* ctx, const meso_scene* const* scenes, const meso_camera* h_cams,
                          uint32_t n_views, const float light[3], uint32_t flags, meso_hit* d_hits,
                          void* stream);
/* The plain form: one launch per view. */
meso_status meso_raymarch_per_view(meso_ctx* ctx, const meso_scene* const* scenes,
                                   const meso_camera* h_cams, uint32_t n_views, const float light[3],
                                   uint32_t flags, meso_hit* d_hits, void* stream);
/* Host-buffer form: the hits land in h_hits when the call returns.  When
 * h_hits is page-locked and device-mapped (meso_host_alloc_pinned, or
 * cudaHostRegister with mapping), the kernel writes the hits straight into
 * it, overlapped with the tracing; otherwise they go through a device buffer
 * and one copy. */
meso_status meso_raymarch_host(meso_ctx* ctx, const meso_scene* scene, const meso_camera* h_cam,
                               const float light[3], uint32_t flags, meso_hit* h_hits);

/* Same launch and results as meso_raymarch (at most 32 views) through a
 * separate kernel instantiation that takes every brick step (no cell jumps)
 * and counts, over all primary and shadow rays: h_counts[0] brick-pointer
 * fetches, [1] occupied bricks entered, [2] hits, [3] rays.  For roofline
 * accounting; the timed path carries no counters. */
meso_status meso_raymarch_stats(meso_ctx* ctx, const meso_scene* const* scenes, const meso_camera* h_cams,
                                uint32_t n_views, const float light[3], uint32_t flags, meso_hit* d_hits,
                                uint64_t h_counts[4]);

/* Multi-view raymarch that allocates no memory.  No counterpart in the
 * reference (it has no raymarcher); same launch and results as
 * meso_raymarch.  For callers that cannot allocate device memory during the
 * call -- a frame loop on a fixed device-memory budget that must not
 * allocate mid-frame (an allocation can synchronise the device and stall the
 * frame), or a host application whose own memory manager owns all device
 * memory -- the view descriptors go to a fixed device array of 512 x 152
 * bytes (76 KiB) instead of a per-call allocation; they travel there as
 * kernel parameters, 64 views at a time (9.5 KiB of the caller's stack).
 * At most 512 views per call (more returns MESO_ERR_INVALID_ARG).  The array
 * stays resident on every device that loads the library until the process
 * exits.  The calling thread's current device must be the context's device
 * (else MESO_ERR_INVALID_ARG).  The first call on a device looks up the
 * array's address and caches it; make that first call before any stream
 * capture.  All calls share the array: calls whose kernels overlap on the
 * GPU race on it, so keep them on one stream or order them. */
meso_status meso_raymarch_noalloc(meso_ctx* ctx, const meso_scene* const* scenes, const meso_camera* h_cams,
                                  uint32_t n_views, const float light[3], uint32_t flags, meso_hit* d_hits,
                                  void* stream);

/* ------------------------------------------------------------- mesh store */

/* The resident mesh of a brick-map scene: every chunk's quads in one device
 * arena, found through a per-chunk segment table, and replaced chunk by chunk
 * when edits dirty them.  Stands in for the reference's pooled chunk output:
 * slot allocation and replacement in FChunkPool::PushToPool
 * (Runtimes/Voxel/Chunk/ChunkPool.h:446-622), the per-chunk block instances
 * written by PushToBlockPool (:381-445) and their upload for drawing
 * (:653-679).  Quads in the arena are the packed format above with the chunk
 * field cleared (the segment names the chunk); their order inside a segment
 * is unspecified.  A store reads its scene, which must outlive it. */
typedef struct meso_mesh_store meso_mesh_store;

typedef struct meso_mesh_store_info {
  uint64_t n_chunks;             /* (nx/32)(ny/32)(nz/32), chunk c = x + CX*(y + CY*z) */
  uint64_t live_quads;           /* quads held in all segments */
  uint64_t arena_quads;          /* arena capacity */
  uint64_t arena_used;           /* bump pointer: segments (with slack) + replaced ones */
  uint64_t compactions;          /* times the arena was repacked */
  const uint64_t* d_arena;       /* device arena */
  const uint64_t* d_seg_offset;  /* per chunk: first quad (UINT64_MAX: none) */
  const uint32_t* d_seg_count;   /* per chunk: quads */
} meso_mesh_store_info;

/* Meshes every non-empty chunk of the scene into a new store (waits). */
meso_status meso_mesh_store_create(meso_ctx* ctx, const meso_scene* scene, meso_mesh_store** out);
/* Remeshes the n listed chunks (linear indices, e.g. the dirty list of
 * meso_edit_spheres; repeats are meshed once) in one batched launch and
 * replaces their segments: in
 * place when the new quads fit, else at the arena's end; a full arena is
 * repacked (and grown) before the update completes.  Returns when the store
 * holds the new segments. */
meso_status meso_mesh_store_update(meso_ctx* ctx, meso_mesh_store* store, const uint32_t* h_chunks, uint32_t n);
meso_status meso_mesh_store_get_info(meso_ctx* ctx, const meso_mesh_store* store, meso_mesh_store_info* info);
/* Copies the segments of the n listed chunks (at most 2^20) into d_out in
 * list order; quads of the k-th listed chunk carry chunk field k.
 * *h_total receives the number of quads (MESO_ERR_OVERFLOW when it exceeds
 * capacity).  Waits for the copy. */
meso_status meso_mesh_store_gather(meso_ctx* ctx, const meso_mesh_store* store, const uint32_t* h_chunks, uint32_t n,
                                   uint64_t* d_out, uint64_t capacity, uint64_t* h_total);
meso_status meso_mesh_store_destroy(meso_ctx* ctx, meso_mesh_store* store);

/* ------------------------------------------------------------------- edits */

typedef struct meso_sphere_edit {
  int32_t center[3];
  int32_t radius;
  uint16_t material; /* 0 removes */
  uint16_t pad;
} meso_sphere_edit;

/* Applies spheres in order (the last sphere covering a voxel decides it),
 * allocating bricks from the pool's spare slots and unlinking bricks that
 * become empty.  Writes the sorted linear indices of the dirty 32^3 chunks
 * (chunks meeting a sphere's box grown by one voxel) to h_dirty.
 * Replaces the reference's regenerate-and-repush of whole chunks
 * (Runtimes/Voxel/Chunk/ChunkPool.h:446-622). Stream-ordered; returns after
 * the dirty list is known (host-side), the device work stays asynchronous. */
meso_status meso_edit_spheres(meso_ctx* ctx, meso_scene* scene, const meso_sphere_edit* h_spheres,
                              uint32_t n, uint32_t* h_dirty, uint32_t dirty_capacity, uint32_t* n_dirty,
                              void* stream);

/* ----------------------------------------------------------------- serving */

typedef struct meso_server meso_server;

typedef enum meso_request_kind { MESO_REQ_RENDER = 0, MESO_REQ_EDIT_REMESH_RENDER = 1 } meso_request_kind;

typedef struct meso_request {
  uint32_t kind;            /* meso_request_kind */
  uint32_t scene_index;     /* index into the server's scene table */
  meso_camera camera;
  uint32_t flags;           /* MESO_RAY_SHADOW */
  uint32_t n_edits;
  const meso_sphere_edit* edits; /* copied at submit */
  uint64_t user_tag;
  meso_hit* dst_hits;       /* optional caller-owned destination of the request's
                               width*height hits, reported complete after they land.
                               Device memory of the server's device or page-locked
                               host memory, 8-byte aligned: the raymarch kernel
                               stores into it directly.  Anything else (pageable
                               memory, unaligned, or a keep_hits server): one copy
                               from the batch buffer.  Resolved at submit; the
                               buffer must stay valid until the completion. */
} meso_request;

typedef struct meso_completion {
  uint64_t request_id;
  uint64_t user_tag;
  int32_t status;           /* meso_status of the request */
  uint32_t n_dirty_chunks;
  uint64_t n_quads;
  uint64_t n_rays;          /* primary + shadow rays traced */
  double submit_s, start_s, done_s; /* seconds on the server clock */
  uint64_t hit_checksum;    /* order-sensitive hash of the hit buffer */
  uint64_t quad_checksum;   /* order-insensitive hash of the quads */
} meso_completion;

typedef struct meso_server_config {
  uint32_t max_inflight_batches;  /* concurrent batches (CUDA streams), 0 = 4 */
  uint32_t max_batch_requests;    /* requests per launch, 0 = 64 */
  uint64_t max_batch_rays;        /* primary rays per launch, 0 = 16M */
  uint64_t hbm_budget_bytes;      /* 0 = the context budget */
  uint32_t keep_hits;             /* 1 = copy hits back (meso_server_fetch_hits) */
  uint32_t max_queue;             /* queued requests beyond this are rejected, 0 = no bound */
  float light[3];                 /* direction towards the light (0,0,0 = normalize(0.3,0.5,0.8)) */
  uint64_t max_edit_quads;        /* quad buffer of a remesh, 0 = 16M */
  uint32_t keep_meshes;           /* 1 = keep a mesh store per scene (created at server
                                     creation), updated by every edit request's remesh */
  uint32_t reserved;
} meso_server_config;

/* The serving loop replaces the host ThreadPool + TDoubleBufferQueue pair
 * (Runtimes/Thread/ThreadPool.h:7-127, Runtimes/Thread/DoubleBufferQueue.h:4-51)
 * with a native scheduler thread that admits requests against the HBM
 * budget and batches them onto a pool of CUDA streams as they arrive. */
meso_status meso_server_create(meso_ctx* ctx, const meso_server_config* cfg, meso_scene* const* scenes,
                               uint32_t n_scenes, meso_server** out);
meso_status meso_server_submit(meso_server* srv, const meso_request* req, uint64_t* request_id);
/* Moves up to max finished completions into out (non-blocking). */
meso_status meso_server_poll(meso_server* srv, meso_completion* out, uint32_t max, uint32_t* n);
/* Copies the hits of a finished request (keep_hits = 1) and releases them. */
meso_status meso_server_fetch_hits(meso_server* srv, uint64_t request_id, meso_hit* h_hits, uint64_t capacity);
/* The mesh store the server keeps for scene scene_index (keep_meshes = 1);
 * owned by the server.  Read it only while no edit of that scene is in
 * flight (e.g. after meso_server_drain). */
meso_status meso_server_get_store(meso_server* srv, uint32_t scene_index, meso_mesh_store** out);
meso_status meso_server_drain(meso_server* srv, double timeout_s);
double meso_server_now(const meso_server* srv);
meso_status meso_server_destroy(meso_server* srv);

/* ------------------------------------------------------------- downstream */

/* Brick-map file: 32-byte header {char magic[8] = "MESOBRK1", uint32 version = 1,
 * int32 nx, ny, nz, uint32 reserved, uint64 n_bricks}, then the pointer grid
 * (uint32, live bricks renumbered 0..n-1 in pointer-grid order, the order a
 * fresh build uses), then n occupancy masks (8 x uint64) and n material
 * bricks (512 x uint16); little endian.  Lets resident scenes be saved and
 * reloaded for reproducible serving runs (the reference regenerates chunks
 * procedurally and has no scene file). */
meso_status meso_scene_save(meso_ctx* ctx, const meso_scene* scene, const char* path);
meso_status meso_scene_load(meso_ctx* ctx, const char* path, uint64_t spare_bricks, meso_scene** out);

/* Vertex of an expanded quad: world position in voxel units and
 * attr = material | dir << 16 | corner << 19. */
typedef struct meso_vertex {
  float x, y, z;
  uint32_t attr;
} meso_vertex;

/* Expands n packed quads into 4 vertices each, counter-clockwise seen from
 * outside the face; a quad of chunk index c sits at chunk_origin[c]*32 (int32
 * triples, device).  The step after meshing for a raster consumer; replaces
 * the reference's per-block FGPUBlock instance stream
 * (Runtimes/Voxel/Block/Block.h:21-65) and the corner placement of its
 * imposter vertex shader (Samples/SimpleVoxel.cpp:171-189).  d_out must be
 * 16-byte aligned. */
meso_status meso_quads_to_vertices(meso_ctx* ctx, const uint64_t* d_quads, uint64_t n_quads,
                                   const int32_t* d_chunk_origins, uint32_t n_chunks, meso_vertex* d_out,
                                   void* stream);

/* The reference's occupancy erosion pyramid on 32^3 chunks
 * (FChunk::CalculateOccupancyErodeMipmaps, Runtimes/Voxel/Chunk/Chunk.h:73-94,
 * with FOccupancyHelper::ErodeSingleVoxel,
 * Runtimes/Voxel/Occupancy/BinaryOccupancyVolume.h:76-99): mip 0 is the
 * occupancy; a voxel is set in mip d >= 1 iff it is set in mip 0, lies at
 * least one voxel inside the chunk border, and all 26 neighbours are set in
 * mip d-1.  d_out receives n * depth * 1024 uint32 words: chunk, mip, word
 * (z, y) with bit x.  depth in 1..8.  The reference culls a block when mip 1
 * has it set (Runtimes/Voxel/Chunk/ChunkPool.h:387). */
meso_status meso_erode_mips(meso_ctx* ctx, const meso_mesh_source* src, const int32_t* d_chunk_coords,
                            uint32_t n_chunks, uint32_t depth, uint32_t* d_out, void* stream);

/* ------------------------------------------------------------------ graphs */

/* CUDA-graph capture of a sequence of stream-ordered meso calls (meshing,
 * raymarching, memset/copy helpers) issued on `stream` between begin and end;
 * meso_graph_launch replays it with one launch.  Calls that wait for the
 * device (meso_sync, meso_mesh_check, scene creation, edits, the host-buffer
 * forms) must not be issued while capturing.  A captured mesh launch keeps
 * the queue ticket it was given; replays of one graph must not overlap each
 * other on different streams. */
typedef struct meso_graph meso_graph;
meso_status meso_capture_begin(meso_ctx* ctx, void* stream);
meso_status meso_capture_end(meso_ctx* ctx, void* stream, meso_graph** out);
meso_status meso_graph_launch(meso_graph* graph, void* stream);
meso_status meso_graph_destroy(meso_graph* graph);

/* ------------------------------------------------------------------ tuning */

/* Grid search on synthetic inputs, standing in for the hand-set
 * ChunkTaskPerCore / MaxUnsyncedLoadChunkCount (Runtimes/Voxel/VoxelSceneConfig.h:35-37):
 * the ray tile shape (lanes along x, warps per CTA) on a 1280x720 view of a
 * 512^3 terrain, and the mesher's CTAs per SM (1 or 2; a CTA meshes one
 * 32^3 chunk = 64 bricks at a time, so this sets the bricks in flight per
 * SM) and chunks per queue ticket on 1024 generated chunks.  Applies the
 * fastest to ctx and writes flat JSON to path (NULL = do not write), which
 * meso_config.tuning_path reads back. */
meso_status meso_autotune(meso_ctx* ctx, const char* path);

#ifdef __cplusplus
}
#endif
#endif
