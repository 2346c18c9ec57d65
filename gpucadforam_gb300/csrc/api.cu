// Host side of the C ABI declared in include/gcm.h.
//
// The reference runs every step of an extraction on the legacy default stream
// with a cudaDeviceSynchronize and blocking count readbacks between them
// (src/Isosurface.cu:44-134, :401-486).  Here each call is stream-ordered: the
// counts come back in one copy at the end (or stay on the device for the
// *_async forms), scratch lives in the context and is zeroed with one memset.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/gcm.h"
#include "gcm_ctx.h"
#include "gcm_kernels.h"

using gcm::MeshParams;

namespace {

constexpr size_t kMeshSmemBudget = 96 * 1024;

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

}  // namespace

namespace gcm {

gcm_status fail(gcm_ctx* ctx, gcm_status s, const char* fmt, ...) {
  if (ctx) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    ctx->last_error = buf;
  }
  return s;
}

gcm_status cuda_fail(gcm_ctx* ctx, cudaError_t e, const char* what) {
  if (e == cudaErrorMemoryAllocation) return fail(ctx, GCM_ERR_OUT_OF_MEMORY, "%s: %s", what, cudaGetErrorString(e));
  return fail(ctx, GCM_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}


gcm_status ensure_scratch(gcm_ctx* ctx, size_t bytes) {
  // Growing allocates; under stream capture cudaMalloc fails and the error is
  // returned, so callers that capture reserve first (gcm_ctx_reserve).
  if (bytes <= ctx->scratch_bytes) return GCM_OK;
  if (ctx->lent)
    return fail(ctx, GCM_ERR_OUT_OF_MEMORY, "lent scratch of %zu bytes, %zu needed", ctx->scratch_bytes, bytes);
  if (ctx->scratch) cudaFree(ctx->scratch);
  ctx->scratch = nullptr;
  ctx->scratch_bytes = 0;
  const size_t sz = align_up(bytes + bytes / 4, 1 << 20);
  GCM_CUDA(ctx, cudaMalloc(&ctx->scratch, sz));
  ctx->scratch_bytes = sz;
  return GCM_OK;
}

gcm_status ensure_buffer(gcm_ctx* ctx, float** buf, size_t* have, size_t bytes) {
  if (bytes <= *have) return GCM_OK;
  if (ctx->lent) return fail(ctx, GCM_ERR_OUT_OF_MEMORY, "lent buffer of %zu bytes, %zu needed", *have, bytes);
  if (*buf) cudaFree(*buf);
  *buf = nullptr;
  *have = 0;
  const size_t sz = align_up(bytes, 1 << 20);
  GCM_CUDA(ctx, cudaMalloc(reinterpret_cast<void**>(buf), sz));
  *have = sz;
  return GCM_OK;
}

void count_launch(gcm_ctx* ctx, uint64_t n) { ctx->launches.fetch_add(n, std::memory_order_relaxed); }

gcm_status check_grid(gcm_ctx* ctx, const gcm_grid* g) {
  if (!g) return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "grid is NULL");
  if (g->nx < 2 || g->ny < 2 || g->nz < 2)
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "grid needs at least 2 samples per axis (got %u x %u x %u)", g->nx,
                g->ny, g->nz);
  if (g->nx > 16384 || g->ny > 65536 || g->nz > 65536)
    return fail(ctx, GCM_ERR_NOT_SUPPORTED, "grid %u x %u x %u exceeds the supported extent", g->nx, g->ny, g->nz);
  return GCM_OK;
}

// Tile shape of the fused mesh kernel: R whole voxel rows of about
// ctx->tile_voxels voxels, within the shared-memory budget.
struct MeshPlan {
  uint32_t rows, tiles_per_plane, blocks;
  int threads;
  uint64_t ntiles;
  MeshLayout layout;
};

uint32_t rows_for(uint32_t nx, uint32_t ny, uint32_t tile_voxels) {
  const uint32_t vx = nx - 1;
  return std::min(std::min(std::max<uint32_t>(1, (tile_voxels + vx / 2) / vx), ny - 1), max_tile_rows(vx));
}

gcm_status plan_mesh(gcm_ctx* ctx, const gcm_grid* g, int mode, MeshPlan* out) {
  const uint32_t vy = g->ny - 1, vz = g->nz - 1;
  int threads = ctx->mesh_threads;
  uint32_t tile_voxels = ctx->tile_voxels;
  if (!ctx->shape_set && mode == kMeshBand) {
    // the band form stages two fields; 256 threads x 2048 voxels measured best
    // for it (384^3 and 512^3 band meshes: 5% and 8% under 128 x 1024)
    threads = 256;
    tile_voxels = 2048;
  }
  uint32_t rows = rows_for(g->nx, g->ny, tile_voxels);
  const size_t budget = std::min(kMeshSmemBudget, ctx->smem_optin);
  while (rows > 1 && mesh_layout_for(g->nx, rows, mode, threads).total > budget) --rows;
  const MeshLayout L = mesh_layout_for(g->nx, rows, mode, threads);
  if (L.total > ctx->smem_optin)
    return fail(ctx, GCM_ERR_NOT_SUPPORTED, "grid rows of %u samples do not fit in shared memory", g->nx);
  out->rows = rows;
  out->threads = threads;
  out->tiles_per_plane = (vy + rows - 1) / rows;
  out->ntiles = (uint64_t)out->tiles_per_plane * vz;
  out->layout = L;
  if (out->ntiles >= (1ull << 31)) return fail(ctx, GCM_ERR_NOT_SUPPORTED, "too many tiles");
  out->blocks = 0;
  return GCM_OK;
}

gcm_status launch_mesh_kernel(gcm_ctx* ctx, int mode, bool emit, MeshParams& p, MeshPlan& plan, cudaStream_t st) {
  int per_sm = 0;
  GCM_CUDA(ctx, gcm::mesh_prepare(mode, emit, plan.threads, plan.layout.total, &per_sm));
  per_sm = std::max(per_sm, 1);
  const uint64_t want = (uint64_t)ctx->sm_count * (uint64_t)per_sm;
  plan.blocks = (uint32_t)std::min<uint64_t>(want, plan.ntiles);
  GCM_CUDA(ctx, gcm::launch_mesh(mode, emit, plan.threads, p, plan.layout, plan.blocks, st));
  count_launch(ctx, 1);
  return GCM_OK;
}

// Scratch for one mesh call: [counts 64 B][counter 64 B][tile states].
struct MeshScratch {
  gcm_counts* counts;
  uint32_t* counter;
  uint64_t* status;
  size_t bytes;
};

MeshScratch carve_mesh_scratch(void* base, uint64_t ntiles) {
  MeshScratch s;
  char* b = static_cast<char*>(base);
  s.counts = reinterpret_cast<gcm_counts*>(b);
  s.counter = reinterpret_cast<uint32_t*>(b + 64);
  s.status = reinterpret_cast<uint64_t*>(b + 128);
  s.bytes = 128 + ntiles * sizeof(uint64_t);
  return s;
}

gcm_status status_of(gcm_ctx* ctx, const gcm_counts& c) {
  switch (c.status) {
    case 0: return GCM_OK;
    case GCM_ERR_OUTPUT_OVERFLOW:
      return fail(ctx, GCM_ERR_OUTPUT_OVERFLOW, "output capacity too small: %llu vertices needed",
                  (unsigned long long)c.total_verts);
    case GCM_ERR_DEVICE_TIMEOUT: return fail(ctx, GCM_ERR_DEVICE_TIMEOUT, "a device-side wait exceeded its limit");
    default: return fail(ctx, GCM_ERR_CUDA, "device reported status %u", c.status);
  }
}

// Core of every fused extraction.  counts_out: device pointer receiving the
// counts (the context's scratch when null).  The caller zeroes nothing.
// The sparse path of a plain extraction: window counts, their exclusive scan,
// emission of the windows that hold triangles.  Scratch: [0, 64) counts,
// [64, 68) scan tile counter, [72, 80) scan total, [128, ...) scan tile
// states, then the window counts and their offsets.
struct SparseLayout {
  uint64_t rows, nwin, scan_tiles;
  size_t off_tris, off_off, bytes;
};

SparseLayout sparse_layout(const gcm_grid* grid) {
  SparseLayout L;
  const uint32_t vx = grid->nx - 1, vy = grid->ny - 1, vz = grid->nz - 1;
  L.rows = (uint64_t)vy * vz;
  L.nwin = L.rows * windows_per_row(vx);
  const uint64_t tile = scan_tile_elems();
  L.scan_tiles = (L.nwin + tile - 1) / tile;
  L.off_tris = (128 + L.scan_tiles * 8 + 15) & ~(size_t)15;
  L.off_off = (L.off_tris + L.nwin * 4 + 15) & ~(size_t)15;
  L.bytes = L.off_off + L.nwin * 4;
  return L;
}

gcm_status mesh_sparse(gcm_ctx* ctx, const float* f, const gcm_grid* grid, float iso, float* pos, float* norm,
                       uint64_t capacity, gcm_counts* counts_out, cudaStream_t st, gcm_counts** counts_used,
                       TileStates tiles = {}) {
  const SparseLayout SL = sparse_layout(grid);
  const uint64_t rows = SL.rows, nwin = SL.nwin, scan_tiles = SL.scan_tiles;
  if (scan_tiles >= (1ull << 31)) return fail(ctx, GCM_ERR_NOT_SUPPORTED, "grid too large for the sparse path");
  const size_t off_tris = SL.off_tris, off_off = SL.off_off;
  gcm_status s = ensure_scratch(ctx, SL.bytes);
  if (s) return s;
  char* b = static_cast<char*>(ctx->scratch);
  gcm_counts* cnt = counts_out ? counts_out : reinterpret_cast<gcm_counts*>(b);
  GCM_CUDA(ctx, cudaMemsetAsync(b, 0, 128 + scan_tiles * 8, st));
  if (counts_out) GCM_CUDA(ctx, cudaMemsetAsync(counts_out, 0, sizeof(gcm_counts), st));
  uint32_t* win_tris = reinterpret_cast<uint32_t*>(b + off_tris);
  uint32_t* win_off = reinterpret_cast<uint32_t*>(b + off_off);
  const uint32_t blocks = grid_blocks(ctx, rows * 32, 256, 8);
  GCM_CUDA(ctx, launch_window_count(f, grid->nx, grid->ny, grid->nz, iso, win_tris, cnt, blocks, st, tiles));
  ScanParams sp{};
  sp.in = win_tris;
  sp.out = win_off;
  sp.n = nwin;
  sp.ntiles = scan_tiles;
  sp.tile_status = reinterpret_cast<uint64_t*>(b + 128);
  sp.counter = reinterpret_cast<uint32_t*>(b + 64);
  sp.total = reinterpret_cast<uint64_t*>(b + 72);
  sp.status = &cnt->status;
  sp.wait_ns = ctx->wait_ns;
  GCM_CUDA(ctx, launch_scan(sp, (uint32_t)std::min<uint64_t>(scan_tiles, (uint64_t)ctx->sm_count * 8), st));
  WindowEmitParams ep{};
  ep.f = f;
  ep.nx = grid->nx;
  ep.ny = grid->ny;
  ep.nz = grid->nz;
  for (int a = 0; a < 3; ++a) {
    ep.vs[a] = grid->voxel_size[a];
    ep.gc[a] = grid->grid_center[a];
  }
  ep.iso = iso;
  ep.win_tris = win_tris;
  ep.win_off = win_off;
  ep.pos = reinterpret_cast<float4*>(pos);
  ep.norm = reinterpret_cast<float4*>(norm);
  ep.capacity = capacity;
  ep.status = &cnt->status;
  GCM_CUDA(ctx, launch_window_emit(ep, blocks, st));
  count_launch(ctx, 3);
  if (counts_used) *counts_used = cnt;
  return GCM_OK;
}

gcm_status mesh_core(gcm_ctx* ctx, const float* f, const float* gfield, const gcm_grid* grid, float iso, float lo,
                     float hi, int mode, uint32_t op, bool emit, float* pos, float* norm, uint64_t capacity,
                     gcm_counts* counts_out, cudaStream_t st, gcm_counts** counts_used, bool sparse_scene = false,
                     TileStates tiles = {}) {
  if (((reinterpret_cast<uintptr_t>(pos) | reinterpret_cast<uintptr_t>(norm)) & 15u) != 0)
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "position and normal buffers must be 16-byte aligned");
  if (mode == kMeshPlain && emit &&
      (ctx->mesh_path == GCM_MESH_PATH_SPARSE || (ctx->mesh_path == GCM_MESH_PATH_AUTO && sparse_scene)))
    return mesh_sparse(ctx, f, grid, iso, pos, norm, capacity, counts_out, st, counts_used, tiles);
  MeshPlan plan;
  gcm_status s = plan_mesh(ctx, grid, mode, &plan);
  if (s) return s;
  const size_t need = 128 + plan.ntiles * sizeof(uint64_t);
  s = ensure_scratch(ctx, need);
  if (s) return s;
  MeshScratch sc = carve_mesh_scratch(ctx->scratch, plan.ntiles);
  gcm_counts* cnt = counts_out ? counts_out : sc.counts;
  GCM_CUDA(ctx, cudaMemsetAsync(ctx->scratch, 0, emit ? sc.bytes : 128, st));
  if (counts_out) GCM_CUDA(ctx, cudaMemsetAsync(counts_out, 0, sizeof(gcm_counts), st));
  MeshParams p{};
  p.f = f;
  p.g = gfield ? gfield : f;
  p.nx = grid->nx;
  p.ny = grid->ny;
  p.nz = grid->nz;
  p.rows = plan.rows;
  p.tiles_per_plane = plan.tiles_per_plane;
  p.ntiles = plan.ntiles;
  p.bulk = ((reinterpret_cast<uintptr_t>(f) | reinterpret_cast<uintptr_t>(p.g)) & 15u) == 0;
  for (int a = 0; a < 3; ++a) {
    p.vs[a] = grid->voxel_size[a];
    p.gc[a] = grid->grid_center[a];
  }
  p.iso = iso;
  p.lo = lo;
  p.hi = hi;
  p.op = op;
  p.pos = reinterpret_cast<float4*>(pos);
  p.norm = reinterpret_cast<float4*>(norm);
  p.capacity = capacity;
  p.tile_status = sc.status;
  p.counter = sc.counter;
  p.counts_dev = cnt;
  p.status = &cnt->status;
  p.wait_ns = ctx->wait_ns;
  s = launch_mesh_kernel(ctx, mode, emit, p, plan, st);
  if (counts_used) *counts_used = cnt;
  return s;
}

size_t extraction_scratch_bytes(gcm_ctx* ctx, const gcm_grid* grid, bool sparse) {
  if (!grid || grid->nx < 2 || grid->ny < 2 || grid->nz < 2) return 0;
  if (sparse) return std::max<size_t>(128, sparse_layout(grid).bytes);
  MeshPlan plan;
  if (plan_mesh(ctx, grid, kMeshPlain, &plan) != GCM_OK) return 0;
  return 128 + plan.ntiles * sizeof(uint64_t);
}

gcm_status read_counts(gcm_ctx* ctx, const gcm_counts* d, gcm_counts* h, cudaStream_t st) {
  GCM_CUDA(ctx, cudaMemcpyAsync(ctx->h_pinned, d, sizeof(gcm_counts), cudaMemcpyDeviceToHost, st));
  GCM_CUDA(ctx, cudaStreamSynchronize(st));
  *h = *ctx->h_pinned;
  return status_of(ctx, *h);
}

uint32_t grid_blocks(gcm_ctx* ctx, uint64_t work, uint32_t threads, uint32_t per_sm) {
  const uint64_t want = (work + threads - 1) / threads;
  const uint64_t cap = (uint64_t)ctx->sm_count * per_sm;
  return (uint32_t)std::max<uint64_t>(1, std::min(want, cap));
}

// Row-structured field kernels: one CTA per sample row at a time.
uint32_t row_blocks(gcm_ctx* ctx, uint32_t ny, uint32_t nz) {
  const uint64_t rows = (uint64_t)ny * nz;
  return (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(rows, (uint64_t)ctx->sm_count * 8));
}

}  // namespace gcm

using namespace gcm;

extern "C" {

int gcm_abi_version(void) { return GCM_ABI_VERSION; }

const char* gcm_status_string(gcm_status s) {
  switch (s) {
    case GCM_OK: return "ok";
    case GCM_ERR_INVALID_ARGUMENT: return "invalid argument";
    case GCM_ERR_OUTPUT_OVERFLOW: return "output overflow";
    case GCM_ERR_DEVICE_TIMEOUT: return "device wait timed out";
    case GCM_ERR_CUDA: return "CUDA error";
    case GCM_ERR_OUT_OF_MEMORY: return "out of memory";
    case GCM_ERR_NOT_SUPPORTED: return "not supported";
    case GCM_ERR_IO: return "I/O error";
    case GCM_ERR_REJECTED: return "rejected";
    case GCM_ERR_CANCELLED: return "cancelled";
    case GCM_ERR_BUSY: return "busy";
  }
  return "unknown status";
}

gcm_status gcm_ctx_create(int device, gcm_ctx** out) {
  if (!out) return GCM_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) return GCM_ERR_INVALID_ARGUMENT;
  gcm_ctx* ctx = new gcm_ctx();
  ctx->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
  int optin = 0;
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  ctx->smem_optin = (size_t)optin;
  if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&ctx->h_pinned), sizeof(gcm_counts));
  if (e != cudaSuccess) {
    delete ctx;
    return e == cudaErrorMemoryAllocation ? GCM_ERR_OUT_OF_MEMORY : GCM_ERR_CUDA;
  }
  *out = ctx;
  return GCM_OK;
}

gcm_status gcm_ctx_destroy(gcm_ctx* ctx) {
  if (!ctx) return GCM_OK;
  cudaSetDevice(ctx->device);
  if (ctx->scratch) cudaFree(ctx->scratch);
  if (ctx->field_buf) cudaFree(ctx->field_buf);
  if (ctx->blend_buf) cudaFree(ctx->blend_buf);
  if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
  if (ctx->weld_buf) cudaFree(ctx->weld_buf);
  delete ctx;
  return GCM_OK;
}

const char* gcm_ctx_last_error(const gcm_ctx* ctx) { return ctx ? ctx->last_error.c_str() : ""; }

gcm_status gcm_ctx_reserve(gcm_ctx* ctx, uint64_t max_points) {
  if (!ctx) return GCM_ERR_INVALID_ARGUMENT;
  // one tile holds at least one voxel row; bound tiles by the voxel count
  const size_t need = 128 + (size_t)max_points * sizeof(uint64_t) / 64 + (1 << 16);
  gcm_status s = ensure_scratch(ctx, need);
  if (s) return s;
  return ensure_buffer(ctx, &ctx->field_buf, &ctx->field_bytes, (size_t)max_points * sizeof(float));
}

gcm_status gcm_ctx_set_wait_limit(gcm_ctx* ctx, uint64_t ns) {
  if (!ctx || ns == 0) return GCM_ERR_INVALID_ARGUMENT;
  ctx->wait_ns = ns;
  return GCM_OK;
}

uint64_t gcm_ctx_launch_count(const gcm_ctx* ctx) { return ctx ? ctx->launches.load() : 0; }

gcm_status gcm_ctx_set_mesh_path(gcm_ctx* ctx, gcm_mesh_path path) {
  if (!ctx) return GCM_ERR_INVALID_ARGUMENT;
  if (path != GCM_MESH_PATH_AUTO && path != GCM_MESH_PATH_FUSED && path != GCM_MESH_PATH_SPARSE)
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_ctx_set_mesh_path: unknown path %d", (int)path);
  ctx->mesh_path = path;
  return GCM_OK;
}

gcm_status gcm_ctx_set_primitive_arith(gcm_ctx* ctx, gcm_prim_arith arith) {
  if (!ctx) return GCM_ERR_INVALID_ARGUMENT;
  if (arith != GCM_PRIM_ARITH_DEFAULT && arith != GCM_PRIM_ARITH_REFERENCE)
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_ctx_set_primitive_arith: unknown mode %d", (int)arith);
  ctx->prim_exact = arith == GCM_PRIM_ARITH_REFERENCE;
  return GCM_OK;
}

// ------------------------------------------------------------------ mesh

gcm_status gcm_mesh_field(gcm_ctx* ctx, const float* d_field, const gcm_grid* grid, float iso, float* d_pos,
                          float* d_norm, uint64_t capacity, gcm_counts* h_counts, gcm_stream stream) {
  if (!ctx) return GCM_ERR_INVALID_ARGUMENT;
  if (!d_field || !h_counts || (capacity && (!d_pos || !d_norm)))
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_mesh_field: NULL field, counts or outputs");
  gcm_status s = check_grid(ctx, grid);
  if (s) return s;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  gcm_counts* used = nullptr;
  s = mesh_core(ctx, d_field, nullptr, grid, iso, 0, 0, kMeshPlain, 0, true, d_pos, d_norm, capacity, nullptr, st, &used);
  if (s) return s;
  return read_counts(ctx, used, h_counts, st);
}

gcm_status gcm_mesh_field_async(gcm_ctx* ctx, const float* d_field, const gcm_grid* grid, float iso, float* d_pos,
                                float* d_norm, uint64_t capacity, gcm_counts* d_counts, gcm_stream stream) {
  if (!ctx) return GCM_ERR_INVALID_ARGUMENT;
  if (!d_field || !d_counts || (capacity && (!d_pos || !d_norm)))
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_mesh_field_async: NULL field, counts or outputs");
  gcm_status s = check_grid(ctx, grid);
  if (s) return s;
  return mesh_core(ctx, d_field, nullptr, grid, iso, 0, 0, kMeshPlain, 0, true, d_pos, d_norm, capacity, d_counts,
                   static_cast<cudaStream_t>(stream), nullptr);
}

gcm_status gcm_count_field(gcm_ctx* ctx, const float* d_field, const gcm_grid* grid, float iso, gcm_counts* h_counts,
                           gcm_stream stream) {
  if (!ctx) return GCM_ERR_INVALID_ARGUMENT;
  if (!d_field || !h_counts) return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_count_field: NULL argument");
  gcm_status s = check_grid(ctx, grid);
  if (s) return s;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // the window count kernel: the same counts as the fused kernel's count
  // pass, from one streaming read of the field
  s = ensure_scratch(ctx, 128);
  if (s) return s;
  gcm_counts* cnt = static_cast<gcm_counts*>(ctx->scratch);
  GCM_CUDA(ctx, cudaMemsetAsync(cnt, 0, sizeof(gcm_counts), st));
  const uint64_t rows = (uint64_t)(grid->ny - 1) * (grid->nz - 1);
  GCM_CUDA(ctx, launch_window_count(d_field, grid->nx, grid->ny, grid->nz, iso, nullptr, cnt,
                                    grid_blocks(ctx, rows * 32, 256, 8), st));
  count_launch(ctx, 1);
  return read_counts(ctx, cnt, h_counts, st);
}

gcm_status gcm_mesh_band(gcm_ctx* ctx, const float* d_label, const float* d_norm_field, const gcm_grid* grid, float iso,
                         float lo, float hi, float* d_pos, float* d_norm, uint64_t capacity, gcm_counts* h_counts,
                         gcm_stream stream) {
  if (!ctx) return GCM_ERR_INVALID_ARGUMENT;
  if (!d_label || !d_norm_field || !h_counts || (capacity && (!d_pos || !d_norm)))
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_mesh_band: NULL argument");
  gcm_status s = check_grid(ctx, grid);
  if (s) return s;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  gcm_counts* used = nullptr;
  s = mesh_core(ctx, d_label, d_norm_field, grid, iso, lo, hi, kMeshBand, 0, true, d_pos, d_norm, capacity, nullptr, st, &used);
  if (s) return s;
  return read_counts(ctx, used, h_counts, st);
}

gcm_status gcm_mesh_band_async(gcm_ctx* ctx, const float* d_label, const float* d_norm_field, const gcm_grid* grid,
                               float iso, float lo, float hi, float* d_pos, float* d_norm, uint64_t capacity,
                               gcm_counts* d_counts, gcm_stream stream) {
  if (!ctx) return GCM_ERR_INVALID_ARGUMENT;
  if (!d_label || !d_norm_field || !d_counts || (capacity && (!d_pos || !d_norm)))
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_mesh_band_async: NULL argument");
  gcm_status s = check_grid(ctx, grid);
  if (s) return s;
  return mesh_core(ctx, d_label, d_norm_field, grid, iso, lo, hi, kMeshBand, 0, true, d_pos, d_norm, capacity,
                   d_counts, static_cast<cudaStream_t>(stream), nullptr);
}

// ------------------------------------------------------- retained CSG form

gcm_status gcm_csg_retain(gcm_ctx* ctx, gcm_csg_point* d_acc, const float* d_field, uint32_t nx, uint32_t ny,
                          uint32_t nz, float iso, gcm_csg_op op, gcm_stream stream) {
  if (!ctx) return GCM_ERR_INVALID_ARGUMENT;
  if (!d_acc || !d_field) return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_csg_retain: NULL argument");
  if (op > GCM_CSG_INTERSECT) return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_csg_retain: unknown op %u", (unsigned)op);
  if (nx == 0 || ny == 0 || nz == 0) return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_csg_retain: empty grid");
  const uint64_t n = (uint64_t)nx * ny * nz;
  GCM_CUDA(ctx, launch_csg_retain(d_acc, d_field, nx, ny, nz, iso, (uint32_t)op, false, 0.0f, 0.0f,
                                  grid_blocks(ctx, n, 256), static_cast<cudaStream_t>(stream)));
  count_launch(ctx, 1);
  return GCM_OK;
}

gcm_status gcm_csg_retain_band(gcm_ctx* ctx, gcm_csg_point* d_acc, const float* d_lattice, uint32_t nx, uint32_t ny,
                               uint32_t nz, float iso, float band_lo, float band_hi, gcm_csg_op op,
                               gcm_stream stream) {
  if (!ctx) return GCM_ERR_INVALID_ARGUMENT;
  if (!d_acc || !d_lattice) return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_csg_retain_band: NULL argument");
  if (op > GCM_CSG_INTERSECT)
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_csg_retain_band: unknown op %u", (unsigned)op);
  if (nx == 0 || ny == 0 || nz == 0) return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_csg_retain_band: empty grid");
  const uint64_t n = (uint64_t)nx * ny * nz;
  GCM_CUDA(ctx, launch_csg_retain(d_acc, d_lattice, nx, ny, nz, iso, (uint32_t)op, true, band_lo, band_hi,
                                  grid_blocks(ctx, n, 256), static_cast<cudaStream_t>(stream)));
  count_launch(ctx, 1);
  return GCM_OK;
}

static gcm_status retained_core(gcm_ctx* ctx, const char* who, const gcm_csg_point* d_acc, const float* d_field,
                                gcm_csg_op op, const gcm_grid* grid, float iso, bool emit, float* d_pos,
                                float* d_norm, uint64_t capacity, gcm_counts* h_counts, gcm_stream stream) {
  if (!ctx) return GCM_ERR_INVALID_ARGUMENT;
  if (!d_acc || !h_counts || (emit && capacity && (!d_pos || !d_norm)))
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "%s: NULL accumulator, counts or outputs", who);
  if ((reinterpret_cast<uintptr_t>(d_acc) & 15u) != 0)
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "%s: the accumulator must be 16-byte aligned", who);
  if (op > GCM_CSG_INTERSECT) return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "%s: unknown op %u", who, (unsigned)op);
  gcm_status s = check_grid(ctx, grid);
  if (s) return s;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  gcm_counts* used = nullptr;
  const int mode = d_field ? kMeshPreview : kMeshRegion;
  s = mesh_core(ctx, reinterpret_cast<const float*>(d_acc), d_field, grid, iso, 0, 0, mode, (uint32_t)op, emit,
                emit ? d_pos : nullptr, emit ? d_norm : nullptr, emit ? capacity : 0, nullptr, st, &used);
  if (s) return s;
  return read_counts(ctx, used, h_counts, st);
}

gcm_status gcm_mesh_retained(gcm_ctx* ctx, const gcm_csg_point* d_acc, const float* d_field, gcm_csg_op op,
                             const gcm_grid* grid, float iso, float* d_pos, float* d_norm, uint64_t capacity,
                             gcm_counts* h_counts, gcm_stream stream) {
  return retained_core(ctx, "gcm_mesh_retained", d_acc, d_field, op, grid, iso, true, d_pos, d_norm, capacity,
                       h_counts, stream);
}

gcm_status gcm_count_retained(gcm_ctx* ctx, const gcm_csg_point* d_acc, const float* d_field, gcm_csg_op op,
                              const gcm_grid* grid, float iso, gcm_counts* h_counts, gcm_stream stream) {
  return retained_core(ctx, "gcm_count_retained", d_acc, d_field, op, grid, iso, false, nullptr, nullptr, 0,
                       h_counts, stream);
}

gcm_status gcm_mesh_lattice_preview(gcm_ctx* ctx, const gcm_csg_point* d_acc, const float* d_field,
                                    const float* d_lattice, gcm_csg_op op, const gcm_grid* grid, float iso,
                                    float band_lo, float band_hi, float* d_pos, float* d_norm, uint64_t capacity,
                                    gcm_counts* h_counts, gcm_stream stream) {
  static const char* who = "gcm_mesh_lattice_preview";
  if (!ctx) return GCM_ERR_INVALID_ARGUMENT;
  if (!d_lattice || !h_counts || (d_acc != nullptr) == (d_field != nullptr) || (capacity && (!d_pos || !d_norm)))
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT,
                "%s: needs a lattice, counts, and exactly one of the accumulator or a primitive field", who);
  if (d_acc && (reinterpret_cast<uintptr_t>(d_acc) & 15u) != 0)
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "%s: the accumulator must be 16-byte aligned", who);
  if (op > GCM_CSG_INTERSECT) return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "%s: unknown op %u", who, (unsigned)op);
  gcm_status s = check_grid(ctx, grid);
  if (s) return s;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  gcm_counts* used = nullptr;
  const int mode = d_acc ? kMeshLatDynamic : kMeshLatFixed;
  const float* f = d_acc ? reinterpret_cast<const float*>(d_acc) : d_field;
  const bool emit = capacity > 0;
  s = mesh_core(ctx, f, d_lattice, grid, iso, band_lo, band_hi, mode, (uint32_t)op, emit, emit ? d_pos : nullptr,
                emit ? d_norm : nullptr, emit ? capacity : 0, nullptr, st, &used);
  if (s) return s;
  return read_counts(ctx, used, h_counts, st);
}

// ------------------------------------------------------------ staged form

gcm_status gcm_mc_classify(gcm_ctx* ctx, const float* d_field, const gcm_grid* grid, float iso, uint32_t* d_verts,
                           uint32_t* d_occ, uint8_t* d_cube, gcm_stream stream) {
  if (!ctx) return GCM_ERR_INVALID_ARGUMENT;
  if (!d_field) return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_mc_classify: NULL field");
  gcm_status s = check_grid(ctx, grid);
  if (s) return s;
  const uint64_t nvox = (uint64_t)(grid->nx - 1) * (grid->ny - 1) * (grid->nz - 1);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  GCM_CUDA(ctx, gcm::launch_classify(d_field, grid->nx, grid->ny, nvox, iso, d_verts, d_occ, d_cube,
                                      grid_blocks(ctx, nvox, 256), st));
  count_launch(ctx, 1);
  return GCM_OK;
}

gcm_status gcm_scan_exclusive_u32(gcm_ctx* ctx, const uint32_t* d_in, uint32_t* d_out, uint64_t n, uint64_t* h_total,
                                  gcm_stream stream) {
  if (!ctx) return GCM_ERR_INVALID_ARGUMENT;
  if (n == 0) {
    if (h_total) *h_total = 0;
    return GCM_OK;
  }
  if (!d_in || !d_out) return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_scan_exclusive_u32: NULL array");
  const uint64_t tile = scan_tile_elems();
  const uint64_t ntiles = (n + tile - 1) / tile;
  if (ntiles >= (1ull << 31)) return fail(ctx, GCM_ERR_NOT_SUPPORTED, "scan too long");
  gcm_status s = ensure_scratch(ctx, 128 + ntiles * 8);
  if (s) return s;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  char* b = static_cast<char*>(ctx->scratch);
  gcm_counts* cnt = reinterpret_cast<gcm_counts*>(b);
  GCM_CUDA(ctx, cudaMemsetAsync(b, 0, 128 + ntiles * 8, st));
  ScanParams p{};
  p.in = d_in;
  p.out = d_out;
  p.n = n;
  p.ntiles = ntiles;
  p.tile_status = reinterpret_cast<uint64_t*>(b + 128);
  p.counter = reinterpret_cast<uint32_t*>(b + 64);
  p.total = &cnt->total_verts;
  p.status = &cnt->status;
  p.wait_ns = ctx->wait_ns;
  const uint32_t blocks = (uint32_t)std::min<uint64_t>(ntiles, (uint64_t)ctx->sm_count * 8);
  GCM_CUDA(ctx, gcm::launch_scan(p, blocks, st));
  count_launch(ctx, 1);
  if (!h_total) return GCM_OK;
  gcm_counts h{};
  s = read_counts(ctx, cnt, &h, st);
  *h_total = h.total_verts;
  return s;
}

gcm_status gcm_mc_compact(gcm_ctx* ctx, const uint32_t* d_occ, const uint32_t* d_scan, uint64_t n, uint32_t* d_out,
                          gcm_stream stream) {
  if (!ctx) return GCM_ERR_INVALID_ARGUMENT;
  if (n == 0) return GCM_OK;
  if (!d_occ || !d_scan || !d_out) return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_mc_compact: NULL array");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  GCM_CUDA(ctx, gcm::launch_compact(d_occ, d_scan, n, d_out, grid_blocks(ctx, n, 256), st));
  count_launch(ctx, 1);
  return GCM_OK;
}

gcm_status gcm_mc_generate(gcm_ctx* ctx, const float* d_field, const gcm_grid* grid, float iso,
                           const uint32_t* d_compacted, uint64_t active, const uint32_t* d_verts_scan, float* d_pos,
                           float* d_norm, uint64_t capacity, gcm_stream stream) {
  if (!ctx) return GCM_ERR_INVALID_ARGUMENT;
  gcm_status s = check_grid(ctx, grid);
  if (s) return s;
  if (active == 0) return GCM_OK;
  if (!d_field || !d_compacted || !d_verts_scan || !d_pos || !d_norm)
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_mc_generate: NULL argument");
  if (((reinterpret_cast<uintptr_t>(d_pos) | reinterpret_cast<uintptr_t>(d_norm)) & 15u) != 0)
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "position and normal buffers must be 16-byte aligned");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  s = ensure_scratch(ctx, 128);
  if (s) return s;
  gcm_counts* cnt = static_cast<gcm_counts*>(ctx->scratch);
  GCM_CUDA(ctx, cudaMemsetAsync(cnt, 0, sizeof(gcm_counts), st));
  GenerateParams p{};
  p.f = d_field;
  p.g = d_field;
  p.nx = grid->nx;
  p.ny = grid->ny;
  p.nz = grid->nz;
  for (int a = 0; a < 3; ++a) {
    p.vs[a] = grid->voxel_size[a];
    p.gc[a] = grid->grid_center[a];
  }
  p.iso = iso;
  p.compacted = d_compacted;
  p.active = active;
  p.verts_scan = d_verts_scan;
  p.pos = reinterpret_cast<float4*>(d_pos);
  p.norm = reinterpret_cast<float4*>(d_norm);
  p.capacity = capacity;
  p.status = &cnt->status;
  GCM_CUDA(ctx, gcm::launch_generate(false, p, grid_blocks(ctx, active, 128, 16), st));
  count_launch(ctx, 1);
  gcm_counts h{};
  return read_counts(ctx, cnt, &h, st);
}

// ------------------------------------------------------------------ fields

gcm_status gcm_field_unit_cell(gcm_ctx* ctx, uint32_t type, uint32_t nx, uint32_t ny, uint32_t nz, float* d_out,
                               gcm_stream stream) {
  if (!ctx) return GCM_ERR_INVALID_ARGUMENT;
  if (!d_out || type > 5 || nx < 2 || ny < 2 || nz < 2)
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_field_unit_cell: bad argument");
  const uint64_t n = (uint64_t)nx * ny * nz;
  GCM_CUDA(ctx, gcm::launch_unit_cell(type, nx, ny, nz, d_out, grid_blocks(ctx, n, 256),
                                       static_cast<cudaStream_t>(stream)));
  count_launch(ctx, 1);
  return GCM_OK;
}

static gcm_status lattice_params(gcm_ctx* ctx, const gcm_lattice* L, uint32_t nx, uint32_t ny, uint32_t nz,
                                 LatticeParams* p) {
  if (!L || !L->d_period || !L->d_type) return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "lattice: NULL period or type");
  if (L->cx == 0 || L->cy == 0 || L->cz == 0) return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "lattice: empty control grid");
  if (L->mode > 1) return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "lattice: unknown grading mode %u", L->mode);
  if ((uint64_t)L->cx * L->cy * L->cz > (1u << 24)) return fail(ctx, GCM_ERR_NOT_SUPPORTED, "control grid too large");
  // the field kernels count sample rows (ny * nz) and step through them in 32 bits
  if ((uint64_t)ny * nz >= (1ull << 31))
    return fail(ctx, GCM_ERR_NOT_SUPPORTED, "lattice grid has %llu sample rows (ny * nz), at most 2^31 - 1",
                (unsigned long long)ny * nz);
  *p = LatticeParams{};
  p->mode = L->mode;
  p->cx = L->cx;
  p->cy = L->cy;
  p->cz = L->cz;
  p->period = L->d_period;
  p->euler = L->d_euler;
  p->thickness = L->d_thickness;
  p->type = L->d_type;
  const uint32_t c[3] = {L->cx, L->cy, L->cz}, n[3] = {nx, ny, nz};
  for (int a = 0; a < 3; ++a) {
    p->origin[a] = L->origin[a];
    p->scale[a] = (c[a] > 1 && n[a] > 1) ? (float)(c[a] - 1) / (float)(n[a] - 1) : 0.0f;
    p->anchor[a] = (c[a] > 1) ? (float)(n[a] - 1) / (float)(c[a] - 1) : 0.0f;
  }
  p->nx = nx;
  p->ny = ny;
  p->nz = nz;
  return GCM_OK;
}

static gcm_status run_lattice(gcm_ctx* ctx, LatticeParams& p, float* d_out, cudaStream_t st) {
  p.out = d_out;
  if (p.mode == GCM_GRADE_BLEND) {
    const uint64_t nc = (uint64_t)p.cx * p.cy * p.cz;
    gcm_status s = ensure_buffer(ctx, &ctx->blend_buf, &ctx->blend_bytes, nc * GCM_BLEND_WORDS * sizeof(float));
    if (s) return s;
    GCM_CUDA(ctx, gcm::launch_lattice(p, ctx->blend_buf, grid_blocks(ctx, nc, 256), row_blocks(ctx, p.ny, p.nz),
                                      (uint32_t)ctx->sm_count, st));
    count_launch(ctx, 2);
  } else {
    GCM_CUDA(ctx, gcm::launch_lattice(p, nullptr, 0, row_blocks(ctx, p.ny, p.nz), (uint32_t)ctx->sm_count, st));
    count_launch(ctx, 1);
  }
  return GCM_OK;
}

gcm_status gcm_field_lattice(gcm_ctx* ctx, const gcm_lattice* lattice, uint32_t nx, uint32_t ny, uint32_t nz,
                             float* d_out, gcm_stream stream) {
  if (!ctx) return GCM_ERR_INVALID_ARGUMENT;
  if (!d_out || nx == 0 || ny == 0 || nz == 0) return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_field_lattice: bad output");
  LatticeParams p;
  gcm_status s = lattice_params(ctx, lattice, nx, ny, nz, &p);
  if (s) return s;
  return run_lattice(ctx, p, d_out, static_cast<cudaStream_t>(stream));
}

gcm_status gcm_mesh_lattice(gcm_ctx* ctx, const gcm_lattice* lattice, const gcm_grid* grid, float iso, float* d_pos,
                            float* d_norm, uint64_t capacity, gcm_counts* h_counts, gcm_stream stream) {
  if (!ctx) return GCM_ERR_INVALID_ARGUMENT;
  if (!h_counts || (capacity && (!d_pos || !d_norm)))
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_mesh_lattice: NULL counts or outputs");
  gcm_status s = check_grid(ctx, grid);
  if (s) return s;
  LatticeParams p;
  s = lattice_params(ctx, lattice, grid->nx, grid->ny, grid->nz, &p);
  if (s) return s;
  const uint64_t n = (uint64_t)grid->nx * grid->ny * grid->nz;
  s = ensure_buffer(ctx, &ctx->field_buf, &ctx->field_bytes, n * sizeof(float));
  if (s) return s;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  s = run_lattice(ctx, p, ctx->field_buf, st);
  if (s) return s;
  gcm_counts* used = nullptr;
  s = mesh_core(ctx, ctx->field_buf, nullptr, grid, iso, 0, 0, kMeshPlain, 0, true, d_pos, d_norm, capacity, nullptr, st, &used);
  if (s) return s;
  return read_counts(ctx, used, h_counts, st);
}

gcm_status gcm_mesh_lattice_async(gcm_ctx* ctx, const gcm_lattice* lattice, const gcm_grid* grid, float iso,
                                  float* d_pos, float* d_norm, uint64_t capacity, gcm_counts* d_counts,
                                  gcm_stream stream) {
  if (!ctx) return GCM_ERR_INVALID_ARGUMENT;
  if (!d_counts || (capacity && (!d_pos || !d_norm)))
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_mesh_lattice_async: NULL counts or outputs");
  gcm_status s = check_grid(ctx, grid);
  if (s) return s;
  LatticeParams p;
  s = lattice_params(ctx, lattice, grid->nx, grid->ny, grid->nz, &p);
  if (s) return s;
  const uint64_t n = (uint64_t)grid->nx * grid->ny * grid->nz;
  s = ensure_buffer(ctx, &ctx->field_buf, &ctx->field_bytes, n * sizeof(float));
  if (s) return s;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  s = run_lattice(ctx, p, ctx->field_buf, st);
  if (s) return s;
  return mesh_core(ctx, ctx->field_buf, nullptr, grid, iso, 0, 0, kMeshPlain, 0, true, d_pos, d_norm, capacity,
                   d_counts, st, nullptr);
}

// The CSG field; with tile_state, also each sample tile's state against iso.
static gcm_status field_csg(gcm_ctx* ctx, const gcm_primitive* d_prims, uint32_t n_prims, const gcm_frame* frame,
                            uint32_t nx, uint32_t ny, uint32_t nz, float* d_out, uint8_t* tile_state, float iso,
                            cudaStream_t st) {
  if (!d_prims || !frame || !d_out || n_prims == 0 || nx == 0 || ny == 0 || nz == 0)
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_field_csg: bad argument");
  if (n_prims > 256) return fail(ctx, GCM_ERR_NOT_SUPPORTED, "gcm_field_csg: at most 256 primitives");
  CsgParams p{};
  p.prims = d_prims;
  p.n = n_prims;
  for (int a = 0; a < 3; ++a) {
    p.origin[a] = frame->origin[a];
    p.spacing[a] = frame->spacing[a];
  }
  p.nx = nx;
  p.ny = ny;
  p.nz = nz;
  p.out = d_out;
  p.exact = ctx->prim_exact ? 1u : 0u;
  p.tile_state = tile_state;
  p.iso = iso;
  GCM_CUDA(ctx, gcm::launch_csg(p, (uint32_t)ctx->sm_count, st));
  count_launch(ctx, 1);
  return GCM_OK;
}

gcm_status gcm_field_csg(gcm_ctx* ctx, const gcm_primitive* d_prims, uint32_t n_prims, const gcm_frame* frame,
                         uint32_t nx, uint32_t ny, uint32_t nz, float* d_out, gcm_stream stream) {
  if (!ctx) return GCM_ERR_INVALID_ARGUMENT;
  return field_csg(ctx, d_prims, n_prims, frame, nx, ny, nz, d_out, nullptr, 0.0f, static_cast<cudaStream_t>(stream));
}

// Field into the context's buffer with its tile states, then the extraction:
// on the windowed path the count pass skips the tasks whose tiles all lie on
// one side of the isovalue without reading their samples.
static gcm_status mesh_csg(gcm_ctx* ctx, const gcm_primitive* d_prims, uint32_t n_prims, const gcm_frame* frame,
                           const gcm_grid* grid, float iso, float* d_pos, float* d_norm, uint64_t capacity,
                           gcm_counts* d_counts, cudaStream_t st, gcm_counts** used) {
  gcm_status s = check_grid(ctx, grid);
  if (s) return s;
  const uint64_t n = (uint64_t)grid->nx * grid->ny * grid->nz;
  const uint32_t tx = (grid->nx + GCM_CSG_TILE_X - 1) / GCM_CSG_TILE_X;
  const uint32_t ty = (grid->ny + GCM_CSG_TILE_Y - 1) / GCM_CSG_TILE_Y;
  const uint64_t tiles = (uint64_t)tx * ty * ((grid->nz + GCM_CSG_TILE_Z - 1) / GCM_CSG_TILE_Z);
  // the field, then the tile states after it (16-byte aligned)
  const size_t field_bytes = (n * sizeof(float) + 15) & ~(size_t)15;
  s = ensure_buffer(ctx, &ctx->field_buf, &ctx->field_bytes, field_bytes + tiles);
  if (s) return s;
  uint8_t* tile_state = reinterpret_cast<uint8_t*>(ctx->field_buf) + field_bytes;
  s = field_csg(ctx, d_prims, n_prims, frame, grid->nx, grid->ny, grid->nz, ctx->field_buf, tile_state, iso, st);
  if (s) return s;
  return mesh_core(ctx, ctx->field_buf, nullptr, grid, iso, 0, 0, kMeshPlain, 0, true, d_pos, d_norm, capacity, d_counts,
                   st, used, true, TileStates{tile_state, tx, ty});
}

gcm_status gcm_mesh_csg(gcm_ctx* ctx, const gcm_primitive* d_prims, uint32_t n_prims, const gcm_frame* frame,
                        const gcm_grid* grid, float iso, float* d_pos, float* d_norm, uint64_t capacity,
                        gcm_counts* h_counts, gcm_stream stream) {
  if (!ctx) return GCM_ERR_INVALID_ARGUMENT;
  if (!h_counts || (capacity && (!d_pos || !d_norm)))
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_mesh_csg: NULL counts or outputs");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  gcm_counts* used = nullptr;
  gcm_status s = mesh_csg(ctx, d_prims, n_prims, frame, grid, iso, d_pos, d_norm, capacity, nullptr, st, &used);
  if (s) return s;
  return read_counts(ctx, used, h_counts, st);
}

gcm_status gcm_mesh_csg_async(gcm_ctx* ctx, const gcm_primitive* d_prims, uint32_t n_prims, const gcm_frame* frame,
                              const gcm_grid* grid, float iso, float* d_pos, float* d_norm, uint64_t capacity,
                              gcm_counts* d_counts, gcm_stream stream) {
  if (!ctx) return GCM_ERR_INVALID_ARGUMENT;
  if (!d_counts || (capacity && (!d_pos || !d_norm)))
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_mesh_csg_async: NULL counts or outputs");
  return mesh_csg(ctx, d_prims, n_prims, frame, grid, iso, d_pos, d_norm, capacity, d_counts,
                  static_cast<cudaStream_t>(stream), nullptr);
}

gcm_status gcm_normalise_band(gcm_ctx* ctx, const float* d_field, uint32_t nx, uint32_t ny, uint32_t nz, float lo,
                              float hi, float* d_label, float* d_norm_field, float* h_minmax, gcm_stream stream) {
  if (!ctx) return GCM_ERR_INVALID_ARGUMENT;
  if (!d_field || !d_label || !d_norm_field || nx == 0 || ny == 0 || nz == 0)
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_normalise_band: bad argument");
  gcm_status s = ensure_scratch(ctx, 128);
  if (s) return s;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned int* enc = reinterpret_cast<unsigned int*>(static_cast<char*>(ctx->scratch) + 64);
  const uint64_t n = (uint64_t)nx * ny * nz;
  GCM_CUDA(ctx, gcm::launch_normalise(d_field, nx, ny, nz, enc, lo, hi, d_label, d_norm_field,
                                       grid_blocks(ctx, n, 256, 4), st));
  count_launch(ctx, 3);
  if (h_minmax) {
    unsigned int k[2];
    GCM_CUDA(ctx, cudaMemcpyAsync(k, enc, sizeof(k), cudaMemcpyDeviceToHost, st));
    GCM_CUDA(ctx, cudaStreamSynchronize(st));
    for (int i = 0; i < 2; ++i) {
      const unsigned int u = (k[i] & 0x80000000u) ? (k[i] & 0x7fffffffu) : ~k[i];
      std::memcpy(&h_minmax[i], &u, 4);
    }
  }
  return GCM_OK;
}

gcm_status gcm_normalise_range(gcm_ctx* ctx, const float* d_in, float* d_out, uint64_t n, float range_lo,
                               float range_span, float* h_minmax, gcm_stream stream) {
  if (!ctx) return GCM_ERR_INVALID_ARGUMENT;
  if (!d_in || !d_out || n == 0) return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_normalise_range: bad argument");
  gcm_status s = ensure_scratch(ctx, 128);
  if (s) return s;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned int* enc = reinterpret_cast<unsigned int*>(static_cast<char*>(ctx->scratch) + 64);
  GCM_CUDA(ctx, gcm::launch_normalise_range(d_in, d_out, n, enc, range_lo, range_span,
                                             grid_blocks(ctx, (n + 3) / 4, 256, 4), st));
  count_launch(ctx, 3);
  if (h_minmax) {
    unsigned int k[2];
    GCM_CUDA(ctx, cudaMemcpyAsync(k, enc, sizeof(k), cudaMemcpyDeviceToHost, st));
    GCM_CUDA(ctx, cudaStreamSynchronize(st));
    for (int i = 0; i < 2; ++i) {
      const unsigned int u = (k[i] & 0x80000000u) ? (k[i] & 0x7fffffffu) : ~k[i];
      std::memcpy(&h_minmax[i], &u, 4);
    }
  }
  return GCM_OK;
}

gcm_status gcm_lattice_mask(gcm_ctx* ctx, const gcm_csg_point* d_acc, const float* d_primitive, float* d_lattice,
                            uint32_t nx, uint32_t ny, uint32_t nz, int fixed, int dynamic, gcm_stream stream) {
  if (!ctx) return GCM_ERR_INVALID_ARGUMENT;
  if (!d_lattice || nx == 0 || ny == 0 || nz == 0 || (fixed && !d_acc) || (!fixed && dynamic && !d_primitive))
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_lattice_mask: bad argument");
  if (!fixed && !dynamic) return GCM_OK;  // the reference's kernel changes nothing then
  const uint64_t n = (uint64_t)nx * ny * nz;
  GCM_CUDA(ctx, gcm::launch_lattice_mask(d_acc, d_primitive, d_lattice, n, fixed != 0, grid_blocks(ctx, n, 256, 4),
                                          static_cast<cudaStream_t>(stream)));
  count_launch(ctx, 1);
  return GCM_OK;
}

gcm_status gcm_test_lookback_stall(gcm_ctx* ctx, uint32_t ntiles, uint32_t stall_tile, uint64_t wait_ns,
                                   uint64_t* d_prefix_out, gcm_stream stream) {
  if (!ctx) return GCM_ERR_INVALID_ARGUMENT;
  if (!d_prefix_out || ntiles == 0 || ntiles > (1u << 20) || wait_ns == 0 || wait_ns > 10000000000ull)
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_test_lookback_stall: bad argument");
  gcm_status s = ensure_scratch(ctx, 128 + (size_t)ntiles * 8);
  if (s) return s;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  char* b = static_cast<char*>(ctx->scratch);
  GCM_CUDA(ctx, cudaMemsetAsync(b, 0, 128 + (size_t)ntiles * 8, st));
  gcm_counts* cnt = reinterpret_cast<gcm_counts*>(b);
  const uint32_t blocks = std::min<uint32_t>(ntiles, (uint32_t)ctx->sm_count * 4);
  GCM_CUDA(ctx, gcm::launch_lookback_stall(ntiles, stall_tile, wait_ns, reinterpret_cast<uint64_t*>(b + 128),
                                           reinterpret_cast<uint32_t*>(b + 64), d_prefix_out, &cnt->status, blocks,
                                           st));
  count_launch(ctx, 1);
  gcm_counts h{};
  return read_counts(ctx, cnt, &h, st);
}

}  // extern "C"
