// Kernel parameter blocks and launch entry points shared by the host library
// (api.cpp) and the CUDA translation units.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "../../include/gcm.h"

// Default launch shape of the fused kernel: CTA size (128 or 256) and the
// voxels per tile it aims for (whole voxel rows of one z-plane).
#ifndef GCM_MESH_THREADS
#define GCM_MESH_THREADS 128
#endif
#ifndef GCM_MESH_TILE_VOXELS
#define GCM_MESH_TILE_VOXELS 1024
#endif
// Triangle-list entries per two voxels of a tile: a tile with more triangles
// emits in several rounds.
#ifndef GCM_MESH_LIST_PER_2VOX
#define GCM_MESH_LIST_PER_2VOX 3
#endif

namespace gcm {

// Extraction modes of the fused kernel: plain (field < iso), band (label
// field + normalised field), and the two meshes of a retained primitive
// accumulator (gcm_csg_point): its region alone, or its preview combined
// with a fed primitive field.
// The lattice previews of the retained editor: a primitive field with a lattice
// band ("fixed"), or the accumulator with a lattice band ("dynamic").
enum MeshMode : int {
  kMeshPlain = 0,
  kMeshBand = 1,
  kMeshRegion = 2,
  kMeshPreview = 3,
  kMeshLatFixed = 4,
  kMeshLatDynamic = 5
};
__host__ __device__ constexpr bool mode_has_g(int mode) {
  return mode == kMeshBand || mode == kMeshPreview || mode == kMeshLatFixed || mode == kMeshLatDynamic;
}
// floats per sample of the classify input (accumulator records are 4 words)
__host__ __device__ constexpr uint32_t mode_fw(int mode) {
  return (mode == kMeshRegion || mode == kMeshPreview || mode == kMeshLatDynamic) ? 4u : 1u;
}
// edges run from the lower corner and carry the stored fraction's offset
__host__ __device__ constexpr bool mode_lower_edges(int mode) { return mode_fw(mode) == 4u; }
// generateTriangles_lattice_kernel's normals: calcNormal(v0, v2, v1), w = 0.5
__host__ __device__ constexpr bool mode_retained_normal(int mode) { return mode >= kMeshRegion; }

// Most voxels in one tile (the triangle list keeps a voxel's index within its
// tile in 16 bits), as a row limit for rows of vx voxels.
constexpr uint32_t kMaxTileVoxels = 65535;
inline uint32_t max_tile_rows(uint32_t vx) { return vx >= kMaxTileVoxels ? 1u : kMaxTileVoxels / vx; }

struct MeshParams {
  const float* f;  // classify field (band mode: the label field)
  const float* g;  // band mode: normalised field used for vertex positions
  uint32_t nx, ny, nz;
  uint32_t rows;             // voxel rows per tile
  uint32_t tiles_per_plane;  // ceil((ny-1) / rows)
  uint32_t bulk;             // 1: stage rows with bulk copies (field bases 16-byte aligned)
  uint64_t ntiles;
  float vs[3], gc[3];
  float iso, lo, hi;
  uint32_t op;            // preview mode: gcm_csg_op combining accumulator and field
  float4* pos;
  float4* norm;
  uint64_t capacity;
  uint64_t* tile_status;  // ntiles words, zeroed before the launch
  uint32_t* counter;      // zeroed before the launch
  gcm_counts* counts_dev; // zeroed before the launch
  uint32_t* status;       // &counts_dev->status
  uint64_t wait_ns;
};

// Shared-memory layout of the fused kernel (computed on the host for the
// largest tile the launch will see).
struct MeshLayout {
  uint32_t plane_stride;  // floats between consecutive staged planes
  uint32_t list_cap;      // triangle-list entries per emission round
  uint32_t f_off, cube_off, win_off, edge_off, list_off, xpose_off, bar_off, total;
};

// One grid of a batched extraction.
struct BatchInstance {
  const float* f;  // field (16-byte aligned when bulk)
  uint32_t nx, ny, nz;
  uint32_t rows, tiles_per_plane, bulk;
  uint64_t tile_begin;  // first tile in the batch's tile sequence
  float vs[3], gc[3];
  float iso;
  uint32_t pad;
};

struct BatchMeshParams {
  const BatchInstance* inst;
  uint32_t n_inst;
  uint64_t ntiles;
  float4* pos;
  float4* norm;
  uint64_t capacity;
  uint64_t* tile_status;
  uint32_t* counter;
  uint32_t* status;
  uint64_t wait_ns;
  uint64_t* offsets;      // n_inst + 1 vertex offsets (emit pass)
  uint64_t* inst_active;  // n_inst active-voxel counts
  uint64_t* inst_verts;   // n_inst vertex counts (count pass)
  gcm_counts* counts_dev; // whole-batch totals and status
};

struct GenerateParams {
  const float* f;
  const float* g;
  uint32_t nx, ny, nz;
  float vs[3], gc[3];
  float iso, lo, hi;
  const uint32_t* compacted;
  uint64_t active;
  const uint32_t* verts_scan;
  float4* pos;
  float4* norm;
  uint64_t capacity;
  uint32_t* status;
};

// Sparse path: windows of 31 voxels of a row, windows_per_row(nx - 1) per row.
__host__ __device__ constexpr uint32_t windows_per_row(uint32_t vx) { return (vx + 30u) / 31u; }

// Sparse path emission: window triangle counts and their exclusive scan.
struct WindowEmitParams {
  const float* f;
  uint32_t nx, ny, nz;
  float vs[3], gc[3];
  float iso;
  const uint32_t* win_tris;
  const uint32_t* win_off;
  float4* pos;
  float4* norm;
  uint64_t capacity;
  uint32_t* status;
};

struct ScanParams {
  const uint32_t* in;
  uint32_t* out;
  uint64_t n;
  uint64_t ntiles;
  uint64_t* tile_status;
  uint32_t* counter;
  uint64_t* total;
  uint32_t* status;
  uint64_t wait_ns;
};

// Words per control point of the blend-mode setup buffer.
#define GCM_BLEND_WORDS 20

// Graded lattice, device form of gcm_lattice.
struct LatticeParams {
  uint32_t mode;
  uint32_t cx, cy, cz;
  const float* period;
  const float* euler;  // [3][n] or null
  const float* thickness;
  const uint8_t* type;
  const float* blend;  // blend mode: per control point GCM_BLEND_WORDS words (R * 2/period as float pairs,
                       // thickness, type)
  float origin[3];
  float scale[3];   // control coordinate per voxel: (c-1)/(n-1)
  float anchor[3];  // voxel spacing of control points: (n-1)/(c-1)
  uint32_t nx, ny, nz;
  float* out;
};

// One graded lattice of a batch (GCM_GRADE_PARAMS), its sample rows starting
// at row_begin of the batch's row sequence.
#define GCM_BATCH_WARP_CX 32  // control columns a warp stages per row

// One instance of the batched field kernel: its sample rows are taken in
// groups of `group_rows` consecutive rows (32 / cx for a staged instance, at
// most 8; 1 for a wide one); group_begin is the first group's index in the
// batch's group sequence.
struct BatchLattice {
  LatticeParams p;
  uint64_t group_begin;
  uint32_t group_rows;
  uint32_t pad;
};
// Rows per group of an instance with cx control columns.
inline uint32_t batch_group_rows(uint32_t cx) {
  if (cx > GCM_BATCH_WARP_CX) return 1;
  const uint32_t r = GCM_BATCH_WARP_CX / cx;
  return r > 8 ? 8 : r;
}

// Sample tile of one warp of the CSG field kernel: 32 along x, 8 rows, 8 planes.
#define GCM_CSG_TILE_X 32
#define GCM_CSG_TILE_Y 8
#define GCM_CSG_TILE_Z 8
// Per-tile state the CSG field kernel can record for the extraction: whether
// every sample of the tile is inside (f < iso), outside, or unknown.
enum : uint8_t { kTileMixed = 0, kTileInside = 1, kTileOutside = 2 };

struct CsgParams {
  const gcm_primitive* prims;
  uint32_t n;
  float origin[3], spacing[3];
  uint32_t nx, ny, nz;
  float* out;
  uint32_t exact;        // GCM_PRIM_ARITH_REFERENCE: the reference's powf squares, bit for bit
  uint8_t* tile_state;   // optional: one kTile* per sample tile, tile index bx + tx * (by + ty * bz)
  float iso;             // the isovalue tile_state is judged against
};

// Tile states for the window count kernel (null state: none).
struct TileStates {
  const uint8_t* state;
  uint32_t tx, ty;  // tiles along x and y
};

// Launch wrappers (each kernel is launched from the file that defines it).
bool mesh_threads_supported(int threads);
MeshLayout mesh_layout(uint32_t plane_floats, uint32_t tile_voxels, uint32_t windows, int mode, int threads);
MeshLayout mesh_layout_for(uint32_t nx, uint32_t rows, int mode, int threads);
cudaError_t mesh_prepare(int mode, bool emit, int threads, size_t smem, int* blocks_per_sm);
cudaError_t launch_mesh(int mode, bool emit, int threads, const MeshParams& p, const MeshLayout& L, uint32_t blocks,
                        cudaStream_t st);
cudaError_t batch_prepare(bool emit, int threads, size_t smem, int* blocks_per_sm);
cudaError_t launch_batch_mesh(bool emit, int threads, const BatchMeshParams& p, const MeshLayout& L, uint32_t blocks,
                              cudaStream_t st);
cudaError_t launch_classify(const float* f, uint32_t nx, uint32_t ny, uint64_t nvox, float iso, uint32_t* verts,
                            uint32_t* occ, uint8_t* cube, uint32_t blocks, cudaStream_t st);
cudaError_t launch_compact(const uint32_t* occ, const uint32_t* scan, uint64_t n, uint32_t* out, uint32_t blocks,
                           cudaStream_t st);
cudaError_t launch_generate(bool band, const GenerateParams& p, uint32_t blocks, cudaStream_t st);
cudaError_t launch_scan(const ScanParams& p, uint32_t blocks, cudaStream_t st);
// Sparse path: window counts (win_tris may be null: counts only), then emission.
cudaError_t launch_window_count(const float* f, uint32_t nx, uint32_t ny, uint32_t nz, float iso, uint32_t* win_tris,
                                gcm_counts* counts, uint32_t blocks, cudaStream_t st, TileStates tiles = {});
cudaError_t launch_window_emit(const WindowEmitParams& p, uint32_t blocks, cudaStream_t st);
cudaError_t launch_lookback_stall(uint32_t ntiles, uint32_t stall, uint64_t wait_ns, uint64_t* tile_status,
                                  uint32_t* counter, uint64_t* prefix_out, uint32_t* status, uint32_t blocks,
                                  cudaStream_t st);

cudaError_t launch_unit_cell(uint32_t type, uint32_t nx, uint32_t ny, uint32_t nz, float* out, uint32_t blocks,
                             cudaStream_t st);
// PARAMS mode picks its kernel from the control-grid width (sm_count sizes the
// row groups); blocks is the grid of the blend and unstaged forms.
cudaError_t launch_lattice(const LatticeParams& p, float* blend_buf, uint32_t prep_blocks, uint32_t blocks,
                           uint32_t sm_count, cudaStream_t st);
// Batched lattice fields: one launch for instances with at most
// GCM_BATCH_WARP_CX control columns, a second one only when some are wider.
cudaError_t launch_lattice_batch(const BatchLattice* inst, uint32_t n_inst, uint64_t total_groups, uint32_t blocks,
                                 bool any_wide, cudaStream_t st);
// CSG field over tiles of 32 x 8 x 8 samples, one tile per warp at a time;
// csg_tiles is the CTA count that gives every warp a tile.
uint64_t csg_tiles(uint32_t nx, uint32_t ny, uint32_t nz);
cudaError_t launch_csg(const CsgParams& p, uint32_t sm_count, cudaStream_t st);
cudaError_t launch_normalise(const float* f, uint32_t nx, uint32_t ny, uint32_t nz, unsigned int* enc, float lo,
                             float hi, float* label, float* norm_field, uint32_t blocks, cudaStream_t st);

// Min/max normalisation into [a1, a1 + b1] (in may equal out).
cudaError_t launch_normalise_range(const float* in, float* out, uint64_t n, unsigned int* enc, float a1, float b1,
                                   uint32_t blocks, cudaStream_t st);
// Lattice samples outside the retained model (fixed) or the live primitive
// (otherwise) become FLT_MAX.
cudaError_t launch_lattice_mask(const gcm_csg_point* acc, const float* prim, float* lat, uint64_t n, bool fixed,
                                uint32_t blocks, cudaStream_t st);

size_t mesh_smem_bytes(uint32_t nx, uint32_t rows, int mode);
// Folds one primitive field into a retained accumulator (gcm_csg_point per sample).
cudaError_t launch_csg_retain(gcm_csg_point* acc, const float* f, uint32_t nx, uint32_t ny, uint32_t nz, float iso,
                              uint32_t op, bool band, float iso1, float iso2, uint32_t blocks, cudaStream_t st);
uint32_t scan_tile_elems();

}  // namespace gcm
