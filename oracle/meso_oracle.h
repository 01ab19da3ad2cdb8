/*
 * meso_oracle.h -- CPU oracle for the two MesoEngine voxel hot paths
 * (greedy chunk meshing and two-level brick-map raymarching).
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the correctness checker and the
 * timed CPU baseline.  Only the test suite, the smoke check and the CPU
 * baseline leg of the benchmark may load it.  The product library
 * (mesoengine_gb300) never links, includes or calls anything here.
 *
 * Parity status: UNPINNED by the reference.  The reference MesoEngine has no
 * greedy mesher, no raymarcher and no tests or golden vectors
 * (it emits one imposter cube per surviving block,
 * Runtimes/Voxel/Chunk/ChunkPool.h:381-445, and draws them with a raster
 * vertex shader, Samples/SimpleVoxel.cpp:146-192).  This oracle is therefore
 * a clean-room restatement of the published algorithms the hot path names:
 *   - greedy meshing: M. Lysenko, "Meshing in a Minecraft Game" (2012);
 *   - voxel traversal: J. Amanatides and A. Woo, "A Fast Voxel Traversal
 *     Algorithm for Ray Tracing" (Eurographics 1987), applied at two levels;
 *   - lattice hash: M. Jarzynski and M. Olano, "Hash Functions for GPU
 *     Rendering" (JCGT 2020), pcg3d;
 * kept on the reference's data conventions:
 *   - x-fastest linear index x + y*Rx + z*Rx*Ry
 *     (Runtimes/Helper/VoxelMathHelper.h:73-76);
 *   - chunk -> 8^3 brick -> voxel hierarchy with a brick pointer per brick
 *     (Runtimes/Voxel/VoxelStructure.h:14-15, :30-39; Runtimes/Voxel/Block/Block.h:14-19);
 *   - all-ones "invalid" sentinel for an empty brick pointer
 *     (Runtimes/Voxel/Block/Block.h:16-18, Runtimes/Voxel/Chunk/Chunk.h:29);
 *   - outside the volume reads as empty
 *     (Runtimes/Voxel/Occupancy/BinaryOccupancyVolume.h:29-37, :79-82);
 *   - camera rebased on an integer chunk plus a fractional offset, z-up,
 *     vertical field of view (Runtimes/Instance/VoxelCamera.cpp:42-59,
 *     Runtimes/Instance/VoxelCamera.h:23, Runtimes/Instance/VoxelWindowsInstance.h:22).
 * Known-answer cases (single voxel, full chunk, checkerboard, axis rays) pin
 * the oracle by hand instead; the tests hold them.
 *
 * Floating point: every FP32 expression is written as a fixed sequence of
 * single IEEE operations and the file is compiled with -ffp-contract=off, so
 * results are reproducible bit for bit.
 */
#ifndef MESO_ORACLE_H
#define MESO_ORACLE_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MO_EMPTY_BRICK 0xFFFFFFFFu
#define MO_CHUNK 32
#define MO_BRICK 8

/* ---- noise ------------------------------------------------------------ */
uint32_t mo_pcg3d(uint32_t x, uint32_t y, uint32_t z);
float mo_lattice(uint32_t ix, uint32_t iy, uint32_t iz, uint32_t seed);
float mo_vnoise3(uint32_t x, uint32_t y, uint32_t z, uint32_t period, uint32_t seed);
float mo_fbm2(uint32_t x, uint32_t y, uint32_t period, int octaves, uint32_t seed);

/* ---- scene generators -------------------------------------------------- */
/* Dense uint8 grid (the small plain case): 3-octave value noise, periods
 * 64/32/16, amplitudes 1, 1/2, 1/4, normalised by 1.75; solid iff n > 0.5;
 * material = 1 + floor(n*15).  out has nx*ny*nz bytes, x fastest. */
void mo_gen_dense_u8(int nx, int ny, int nz, uint32_t seed, uint8_t* out);

/* Standalone 32^3 uint16 chunks (the batched-meshing case).  Chunk i uses
 * seed seed0+i.  solid_count[i] receives k, the number of solid voxels. */
uint32_t mo_chunk_solid_target(uint32_t seed);
uint32_t mo_chunk_material_count(uint32_t seed);
void mo_gen_chunks_u16(int n_chunks, uint32_t seed0, uint16_t* out, uint32_t* solid_count);

/* Terrain parameters shared by every brick-map scene. */
typedef struct {
  int32_t nx, ny, nz;      /* voxel dims, multiples of 8 */
  uint32_t seed;
  uint32_t height_period;  /* fBm base period (voxels) */
  int32_t height_octaves;
  float height_base;       /* H0 */
  float height_amp;        /* amplitude */
  uint32_t cave_period;    /* 3-D value noise period */
  float cave_threshold;    /* carve where noise > threshold */
} mo_terrain;

float mo_terrain_height(const mo_terrain* t, uint32_t x, uint32_t y);
uint16_t mo_terrain_voxel(const mo_terrain* t, float h, uint32_t x, uint32_t y, uint32_t z);

/* Brick map: ptr has (nx/8)*(ny/8)*(nz/8) entries (x fastest), each a brick
 * index or MO_EMPTY_BRICK; brick b occupies occ[8b..8b+7] (word z, bit
 * x+8y) and mat[512b..512b+511] (index x+8y+64z).  Bricks are numbered in
 * pointer-grid linear order. */
typedef struct {
  int32_t nx, ny, nz;
  uint32_t* ptr;
  uint64_t* occ;
  uint16_t* mat;
  uint64_t n_bricks;
  uint64_t cap_bricks;
} mo_brickmap;

/* Builds the terrain scene.  Returns 0 on success.  Uses nthreads host
 * threads (<=0: all cores).  Arrays are malloc'ed; free with mo_brickmap_free. */
int mo_build_terrain(const mo_terrain* t, int nthreads, mo_brickmap* out);
/* Builds a brick map from a dense uint16 grid (x fastest). */
int mo_build_from_dense_u16(int nx, int ny, int nz, const uint16_t* grid, mo_brickmap* out);
void mo_brickmap_free(mo_brickmap* bm);
uint16_t mo_brickmap_get(const mo_brickmap* bm, int64_t x, int64_t y, int64_t z);
/* Dense uint16 copy of the whole map (for small scenes). */
void mo_brickmap_to_dense(const mo_brickmap* bm, uint16_t* out);

/* ---- greedy meshing ---------------------------------------------------- */
/* Packed quad (uint64), most significant field first:
 *   [63:44] chunk index in the call   [43:41] dir (0 +X,1 -X,2 +Y,3 -Y,4 +Z,5 -Z)
 *   [40:36] z   [35:31] y   [30:26] x  (chunk-local origin voxel)
 *   [25:21] w-1 (along u)   [20:16] h-1 (along v)   [15:0] material
 * Plane axes: X faces u=y v=z; Y faces u=x v=z; Z faces u=x v=y.
 * Sorting the uint64 values numerically is the canonical order
 * (chunk, dir, z, y, x). */
uint64_t mo_pack_quad(uint32_t chunk, int dir, int x, int y, int z, int w, int h, uint16_t mat);

/* Source kinds for the mesher. */
#define MO_SRC_GRID_U8 0     /* dense uint8 grid, neighbours across chunks are real */
#define MO_SRC_CHUNKS_U16 1  /* array of standalone 32^3 uint16 chunks, outside empty */
#define MO_SRC_BRICKMAP 2    /* brick map, neighbours across chunks are real */
#define MO_SRC_GRID_U16 3    /* dense uint16 grid */
#define MO_SRC_CHUNKS_U8 4   /* array of standalone 32^3 uint8 chunks */

typedef struct {
  int kind;
  const void* data;          /* grid / chunk array */
  int32_t nx, ny, nz;        /* grid dims (grid kinds) */
  const mo_brickmap* bm;     /* brick-map kind */
} mo_source;

/* Meshes one chunk.  For chunk-array kinds chunk_coord[0] is the chunk index
 * in the array; for grid/brick-map kinds it is the chunk coordinate.  Writes
 * at most cap quads, returns the number of quads produced (may exceed cap). */
uint64_t mo_mesh_chunk(const mo_source* src, const int32_t chunk_coord[3], uint32_t chunk_id,
                       uint64_t* out, uint64_t cap);
/* Meshes n chunks with nthreads host threads (one chunk per task).  Quads of
 * all chunks are written canonically sorted.  Returns the total count. */
uint64_t mo_mesh_chunks_mt(const mo_source* src, const int32_t* chunk_coords, uint32_t n,
                           int nthreads, uint64_t* out, uint64_t cap);
/* Exposed-face count of one chunk (property checks: sum of quad areas). */
uint64_t mo_count_faces(const mo_source* src, const int32_t chunk_coord[3]);

/* ---- raymarching -------------------------------------------------------- */
typedef struct {
  int32_t origin_chunk[3];  /* camera chunk (32-voxel chunks) */
  float origin_frac[3];     /* position inside that chunk, voxels */
  float forward[3];
  float right[3];
  float up[3];
  float tan_half_fov_y;
  uint32_t width, height;
} mo_camera;

typedef struct {
  uint64_t voxel;     /* x + y*nx + z*nx*ny of the hit voxel; UINT64_MAX on miss */
  float t;            /* distance to the entry of the hit voxel; +inf on miss */
  uint16_t material;
  uint8_t face;       /* entered face normal: 0 +X 1 -X 2 +Y 3 -Y 4 +Z 5 -Z; 6 none */
  uint8_t shadow;     /* 1 occluded, 0 lit, 255 not traced */
  uint32_t steps;     /* primary: fine | coarse << 16 */
  uint32_t shadow_steps;
} mo_hit;

void mo_camera_ray(const mo_camera* cam, uint32_t px, uint32_t py, float dir[3]);
void mo_trace_ray(const mo_brickmap* bm, const int32_t cam_chunk[3], const float o[3],
                  const float d[3], const float light[3], int shadow, mo_hit* hit);
/* Renders n_views cameras; hits laid out view after view, row-major. */
void mo_raymarch_mt(const mo_brickmap* bm, const mo_camera* cams, uint32_t n_views,
                    const float light[3], int shadow, int nthreads, mo_hit* hits);
/* Renders only a subset of rows of one camera (bounded CPU baseline). */
void mo_raymarch_rows_mt(const mo_brickmap* bm, const mo_camera* cam, uint32_t row0,
                         uint32_t n_rows, const float light[3], int shadow, int nthreads,
                         mo_hit* hits);

/* ---- edits -------------------------------------------------------------- */
typedef struct {
  int32_t center[3];
  int32_t radius;
  uint16_t material;  /* 0 = remove */
  uint16_t pad;
} mo_sphere;

/* Applies spheres in order (the last sphere covering a voxel decides it).
 * Grows the brick pool as needed; bricks that become empty are unlinked.
 * Returns 0 on success. */
int mo_edit_spheres(mo_brickmap* bm, const mo_sphere* s, uint32_t n);
/* Dirty 32^3 chunks of an edit list: chunks meeting any sphere's bounding box
 * grown by one voxel, clipped to the grid; written as sorted unique linear
 * chunk indices.  Returns the count. */
uint32_t mo_dirty_chunks(const mo_brickmap* bm, const mo_sphere* s, uint32_t n, uint32_t* out,
                         uint32_t cap);

/* ---- erosion pyramid ----------------------------------------------------- */
/* Restates FChunk::CalculateOccupancyErodeMipmaps (Runtimes/Voxel/Chunk/Chunk.h:73-94)
 * with FOccupancyHelper::ErodeSingleVoxel<true>
 * (Runtimes/Voxel/Occupancy/BinaryOccupancyVolume.h:76-99) on one R^3 chunk
 * (R = 32 here): mip 0 = occupancy; for d >= 1, every voxel of mip 0 is
 * tested: out of the border thickness 1 (VoxelMathHelper.h:106-112) -> 0,
 * else the AND of its 26 Moore neighbours in mip d-1.  occ: R^3 bytes
 * (nonzero = solid, x fastest); out: depth * R^3 bytes. */
void mo_erode_mips(const uint8_t* occ, int R, int depth, uint8_t* out);

int mo_hardware_threads(void);

#ifdef __cplusplus
}
#endif
#endif
