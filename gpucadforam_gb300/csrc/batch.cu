// Batched extraction: many graded lattices of different, non-cubic sizes in
// two launches (all fields, then one persistent fused marching-cubes pass over
// a work list of every instance's tiles), optionally replayed as a CUDA graph,
// with the launch shape picked by an autotuner.
//
// The reference meshes one grid per call, each call a chain of kernels with
// blocking readbacks (src/Isosurface.cu:401-486); a batch of small grids is
// then dominated by launch and synchronisation latency.  Here the instances
// share one tile sequence and one decoupled look-back chain: instance i's
// vertices follow instance i-1's in the output, and each instance's mesh is
// bit for bit the one gcm_mesh_lattice produces for it alone.
//
// Everything a batch needs on the device is allocated by gcm_batch_create and
// by re-planning (gcm_batch_tune); gcm_batch_mesh_async allocates nothing and
// contains no host synchronisation, so it can be captured into a graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gcm.h"
#include "gcm_ctx.h"
#include "gcm_kernels.h"

namespace {

constexpr size_t kSmemBudget = 96 * 1024;

struct Plan {
  int threads = GCM_MESH_THREADS;
  uint32_t tile_voxels = GCM_MESH_TILE_VOXELS;
  uint64_t ntiles = 0;
  gcm::MeshLayout layout{};
  uint32_t blocks_emit = 0, blocks_count = 0;
};

}  // namespace

struct gcm_batch {
  gcm_ctx* ctx = nullptr;
  std::vector<gcm_batch_instance> inst;
  uint32_t n = 0;
  // fields
  float* field = nullptr;
  std::vector<uint64_t> field_off;  // floats, 16-byte aligned starts
  gcm::BatchLattice* d_lat = nullptr;
  uint32_t n_params = 0;  // instances evaluated by the batched field kernel
  uint64_t param_groups = 0;  // row groups of those instances
  bool params_wide = false;  // some instance has more than GCM_BATCH_WARP_CX control columns
  std::vector<uint32_t> blend_ids;  // instances evaluated one by one (blend mode)
  float* blend_buf = nullptr;
  // tiles
  Plan plan;
  gcm::BatchInstance* d_bi = nullptr;
  void* scratch = nullptr;  // [0,64) status + counter, then tile states
  size_t scratch_bytes = 0;
  uint64_t* d_inst = nullptr;  // inst_active[n], inst_verts[n], offsets[n+1] (count pass)
  gcm_counts* d_counts_internal = nullptr;
  // graph
  cudaGraphExec_t exec = nullptr;
  const void* g_key[5] = {};
  uint64_t g_cap = 0;
};

namespace gcm {
namespace {

void free_plan_buffers(gcm_batch* b) {
  if (b->d_bi) cudaFree(b->d_bi);
  b->d_bi = nullptr;
  if (b->scratch) cudaFree(b->scratch);
  b->scratch = nullptr;
  b->scratch_bytes = 0;
}

void drop_graph(gcm_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  b->exec = nullptr;
  std::memset(b->g_key, 0, sizeof(b->g_key));
}

gcm_status make_plan(gcm_batch* b, int threads, uint32_t tile_voxels) {
  gcm_ctx* ctx = b->ctx;
  if (!mesh_threads_supported(threads) || tile_voxels < 64 || tile_voxels > (1u << 20))
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "unsupported launch shape (%d threads, %u voxels)", threads,
                tile_voxels);
  const size_t budget = std::min(kSmemBudget, ctx->smem_optin);
  std::vector<BatchInstance> bi(b->n);
  uint32_t max_plane = 0, max_vox = 0, max_win = 0;
  uint64_t tiles = 0;
  for (uint32_t i = 0; i < b->n; ++i) {
    const gcm_grid& g = b->inst[i].grid;
    const uint32_t vx = g.nx - 1, vy = g.ny - 1, vz = g.nz - 1;
    uint32_t rows = std::min(std::min(std::max<uint32_t>(1, (tile_voxels + vx / 2) / vx), vy), max_tile_rows(vx));
    while (rows > 1 && mesh_layout_for(g.nx, rows, kMeshPlain, threads).total > budget) --rows;
    BatchInstance& I = bi[i];
    I.f = b->field + b->field_off[i];
    I.nx = g.nx;
    I.ny = g.ny;
    I.nz = g.nz;
    I.rows = rows;
    I.tiles_per_plane = (vy + rows - 1) / rows;
    I.bulk = 1;  // field slices start 16-byte aligned
    I.tile_begin = tiles;
    for (int a = 0; a < 3; ++a) {
      I.vs[a] = g.voxel_size[a];
      I.gc[a] = g.grid_center[a];
    }
    I.iso = b->inst[i].iso;
    I.pad = 0;
    tiles += (uint64_t)I.tiles_per_plane * vz;
    max_plane = std::max(max_plane, (rows + 1) * g.nx + 4);
    max_vox = std::max(max_vox, rows * vx);
    max_win = std::max(max_win, rows * ((vx + 31) / 32));
  }
  if (tiles >= (1ull << 31)) return fail(ctx, GCM_ERR_NOT_SUPPORTED, "batch has too many tiles");
  const MeshLayout L = mesh_layout(max_plane, max_vox, max_win, kMeshPlain, threads);
  if (L.total > ctx->smem_optin) return fail(ctx, GCM_ERR_NOT_SUPPORTED, "batch rows do not fit in shared memory");
  drop_graph(b);
  free_plan_buffers(b);
  GCM_CUDA(ctx, cudaMalloc(&b->d_bi, sizeof(BatchInstance) * b->n));
  GCM_CUDA(ctx, cudaMemcpy(b->d_bi, bi.data(), sizeof(BatchInstance) * b->n, cudaMemcpyHostToDevice));
  b->scratch_bytes = 128 + tiles * 8;
  GCM_CUDA(ctx, cudaMalloc(&b->scratch, b->scratch_bytes));
  int pe = 0, pc = 0;
  GCM_CUDA(ctx, batch_prepare(true, threads, L.total, &pe));
  GCM_CUDA(ctx, batch_prepare(false, threads, L.total, &pc));
  Plan p;
  p.threads = threads;
  p.tile_voxels = tile_voxels;
  p.ntiles = tiles;
  p.layout = L;
  p.blocks_emit = (uint32_t)std::min<uint64_t>((uint64_t)ctx->sm_count * std::max(pe, 1), tiles);
  p.blocks_count = (uint32_t)std::min<uint64_t>((uint64_t)ctx->sm_count * std::max(pc, 1), tiles);
  b->plan = p;
  return GCM_OK;
}

gcm_status launch_fields(gcm_batch* b, cudaStream_t st) {
  gcm_ctx* ctx = b->ctx;
  if (b->n_params) {
    // about 2 row groups per warp (8 warps per CTA): many CTAs rather than
    // one resident wave, so the block scheduler balances the SMs
    const uint32_t blocks = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((b->param_groups + 15) / 16, 1u << 26));
    GCM_CUDA(ctx, launch_lattice_batch(b->d_lat, b->n_params, b->param_groups, blocks, b->params_wide, st));
    count_launch(ctx, b->params_wide ? 2 : 1);
  }
  for (uint32_t i : b->blend_ids) {
    const gcm_batch_instance& I = b->inst[i];
    LatticeParams p{};
    p.mode = GCM_GRADE_BLEND;
    p.cx = I.lattice.cx;
    p.cy = I.lattice.cy;
    p.cz = I.lattice.cz;
    p.period = I.lattice.d_period;
    p.euler = I.lattice.d_euler;
    p.thickness = I.lattice.d_thickness;
    p.type = I.lattice.d_type;
    const uint32_t c[3] = {p.cx, p.cy, p.cz}, n[3] = {I.grid.nx, I.grid.ny, I.grid.nz};
    for (int a = 0; a < 3; ++a) {
      p.origin[a] = I.lattice.origin[a];
      p.scale[a] = (c[a] > 1 && n[a] > 1) ? (float)(c[a] - 1) / (float)(n[a] - 1) : 0.0f;
      p.anchor[a] = (c[a] > 1) ? (float)(n[a] - 1) / (float)(c[a] - 1) : 0.0f;
    }
    p.nx = n[0];
    p.ny = n[1];
    p.nz = n[2];
    p.out = b->field + b->field_off[i];
    const uint64_t nc = (uint64_t)p.cx * p.cy * p.cz;
    const uint32_t rows = std::max<uint32_t>(1, std::min<uint32_t>(n[1] * n[2], (uint32_t)ctx->sm_count * 8));
    GCM_CUDA(ctx, launch_lattice(p, b->blend_buf, grid_blocks(ctx, nc, 256), rows, (uint32_t)ctx->sm_count, st));
    count_launch(ctx, 2);
  }
  return GCM_OK;
}

BatchMeshParams mesh_params(gcm_batch* b, float* pos, float* norm, uint64_t cap, uint64_t* offsets,
                            gcm_counts* counts) {
  BatchMeshParams p{};
  p.inst = b->d_bi;
  p.n_inst = b->n;
  p.ntiles = b->plan.ntiles;
  p.pos = reinterpret_cast<float4*>(pos);
  p.norm = reinterpret_cast<float4*>(norm);
  p.capacity = cap;
  char* s = static_cast<char*>(b->scratch);
  p.counter = reinterpret_cast<uint32_t*>(s + 64);
  p.tile_status = reinterpret_cast<uint64_t*>(s + 128);
  p.status = &counts->status;
  p.wait_ns = b->ctx->wait_ns;
  p.offsets = offsets;
  p.inst_active = b->d_inst;
  p.inst_verts = b->d_inst + b->n;
  p.counts_dev = counts;
  return p;
}

// Stream-ordered emit pass: no allocation, no host synchronisation.
gcm_status mesh_async(gcm_batch* b, float* pos, float* norm, uint64_t cap, uint64_t* offsets, gcm_counts* counts,
                      cudaStream_t st) {
  gcm_ctx* ctx = b->ctx;
  GCM_CUDA(ctx, cudaMemsetAsync(b->scratch, 0, b->scratch_bytes, st));
  GCM_CUDA(ctx, cudaMemsetAsync(counts, 0, sizeof(gcm_counts), st));
  GCM_CUDA(ctx, cudaMemsetAsync(b->d_inst, 0, sizeof(uint64_t) * 2 * b->n, st));
  gcm_status s = launch_fields(b, st);
  if (s) return s;
  BatchMeshParams p = mesh_params(b, pos, norm, cap, offsets, counts);
  GCM_CUDA(ctx, launch_batch_mesh(true, b->plan.threads, p, b->plan.layout, b->plan.blocks_emit, st));
  count_launch(ctx, 1);
  return GCM_OK;
}

std::string signature(const gcm_batch* b) {
  uint64_t h = 1469598103934665603ull, pts = 0;
  for (const auto& I : b->inst) {
    for (uint32_t v : {I.grid.nx, I.grid.ny, I.grid.nz, I.lattice.mode}) {
      h ^= v;
      h *= 1099511628211ull;
    }
    pts += (uint64_t)I.grid.nx * I.grid.ny * I.grid.nz;
  }
  char buf[128];
  std::snprintf(buf, sizeof(buf), "n=%u;points=%llu;shape=%016llx", b->n, (unsigned long long)pts,
                (unsigned long long)h);
  return buf;
}

bool cache_lookup(const char* path, const std::string& sig, int* threads, uint32_t* tile_voxels) {
  if (!path) return false;
  FILE* f = std::fopen(path, "r");
  if (!f) return false;
  char line[512];
  bool found = false;
  while (std::fgets(line, sizeof(line), f)) {
    char s[256];
    int t = 0;
    unsigned v = 0;
    double ms = 0;
    if (std::sscanf(line, "gcm-tune-v1 %255s %d %u %lf", s, &t, &v, &ms) == 4 && sig == s) {
      *threads = t;
      *tile_voxels = v;
      found = true;
    }
  }
  std::fclose(f);
  return found;
}

}  // namespace
}  // namespace gcm

using namespace gcm;

extern "C" {

gcm_status gcm_batch_create(gcm_ctx* ctx, const gcm_batch_instance* h_instances, uint32_t n, gcm_batch** out) {
  if (!ctx) return GCM_ERR_INVALID_ARGUMENT;
  if (!out || !h_instances || n == 0) return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_batch_create: bad argument");
  *out = nullptr;
  gcm_batch* b = new gcm_batch();
  b->ctx = ctx;
  b->n = n;
  b->inst.assign(h_instances, h_instances + n);
  b->field_off.resize(n);
  uint64_t off = 0;
  std::vector<BatchLattice> lat;
  std::vector<uint32_t> lat_inst;  // instance of each entry of lat
  uint64_t max_blend_ctrl = 0;
  for (uint32_t i = 0; i < n; ++i) {
    const gcm_batch_instance& I = b->inst[i];
    const gcm_grid& g = I.grid;
    const gcm_lattice& L = I.lattice;
    if (g.nx < 2 || g.ny < 2 || g.nz < 2 || g.nx > 16384 || g.ny > 65536 || g.nz > 65536 || !L.d_period ||
        !L.d_type || L.cx == 0 || L.cy == 0 || L.cz == 0 || L.mode > 1) {
      delete b;
      return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_batch_create: instance %u is invalid", i);
    }
    if ((uint64_t)g.ny * g.nz >= (1ull << 31)) {  // the field kernel counts sample rows in 32 bits
      delete b;
      return fail(ctx, GCM_ERR_NOT_SUPPORTED, "gcm_batch_create: instance %u has too many sample rows", i);
    }
    b->field_off[i] = off;
    off += ((uint64_t)g.nx * g.ny * g.nz + 3) / 4 * 4;
    if (L.mode == GCM_GRADE_BLEND) {
      b->blend_ids.push_back(i);
      max_blend_ctrl = std::max<uint64_t>(max_blend_ctrl, (uint64_t)L.cx * L.cy * L.cz);
      continue;
    }
    BatchLattice bl{};
    LatticeParams& p = bl.p;
    p.mode = 0;
    p.cx = L.cx;
    p.cy = L.cy;
    p.cz = L.cz;
    p.period = L.d_period;
    p.euler = L.d_euler;
    p.thickness = L.d_thickness;
    p.type = L.d_type;
    const uint32_t c[3] = {L.cx, L.cy, L.cz}, nn[3] = {g.nx, g.ny, g.nz};
    for (int a = 0; a < 3; ++a) {
      p.origin[a] = L.origin[a];
      p.scale[a] = (c[a] > 1 && nn[a] > 1) ? (float)(c[a] - 1) / (float)(nn[a] - 1) : 0.0f;
      p.anchor[a] = (c[a] > 1) ? (float)(nn[a] - 1) / (float)(c[a] - 1) : 0.0f;
    }
    p.nx = g.nx;
    p.ny = g.ny;
    p.nz = g.nz;
    if (L.cx > GCM_BATCH_WARP_CX) b->params_wide = true;
    bl.group_begin = b->param_groups;
    bl.group_rows = batch_group_rows(L.cx);
    b->param_groups += ((uint64_t)g.ny * g.nz + bl.group_rows - 1) / bl.group_rows;
    lat.push_back(bl);
    lat_inst.push_back(i);
  }
  b->n_params = (uint32_t)lat.size();
  gcm_status s = GCM_OK;
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&b->field), std::max<uint64_t>(off, 4) * sizeof(float));
  if (e == cudaSuccess) {
    // each instance's slice of the batch field, now that the field exists
    for (size_t k = 0; k < lat.size(); ++k) lat[k].p.out = b->field + b->field_off[lat_inst[k]];
    if (!lat.empty()) e = cudaMalloc(reinterpret_cast<void**>(&b->d_lat), sizeof(BatchLattice) * lat.size());
  }
  if (e == cudaSuccess && !lat.empty())
    e = cudaMemcpy(b->d_lat, lat.data(), sizeof(BatchLattice) * lat.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && max_blend_ctrl)
    e = cudaMalloc(reinterpret_cast<void**>(&b->blend_buf), max_blend_ctrl * GCM_BLEND_WORDS * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&b->d_inst), sizeof(uint64_t) * (3 * (size_t)n + 1));
  if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&b->d_counts_internal), sizeof(gcm_counts));
  if (e != cudaSuccess) s = cuda_fail(ctx, e, "gcm_batch_create allocation");
  if (!s) s = make_plan(b, ctx->mesh_threads, ctx->tile_voxels);
  if (s) {
    gcm_batch_destroy(b);
    return s;
  }
  *out = b;
  return GCM_OK;
}

gcm_status gcm_batch_destroy(gcm_batch* b) {
  if (!b) return GCM_OK;
  drop_graph(b);
  free_plan_buffers(b);
  if (b->field) cudaFree(b->field);
  if (b->d_lat) cudaFree(b->d_lat);
  if (b->blend_buf) cudaFree(b->blend_buf);
  if (b->d_inst) cudaFree(b->d_inst);
  if (b->d_counts_internal) cudaFree(b->d_counts_internal);
  delete b;
  return GCM_OK;
}

gcm_status gcm_batch_count(gcm_batch* b, uint64_t* h_verts, uint64_t* h_active, gcm_counts* h_counts,
                           gcm_stream stream) {
  if (!b) return GCM_ERR_INVALID_ARGUMENT;
  gcm_ctx* ctx = b->ctx;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  gcm_counts* cnt = b->d_counts_internal;
  GCM_CUDA(ctx, cudaMemsetAsync(b->scratch, 0, 128, st));
  GCM_CUDA(ctx, cudaMemsetAsync(cnt, 0, sizeof(gcm_counts), st));
  GCM_CUDA(ctx, cudaMemsetAsync(b->d_inst, 0, sizeof(uint64_t) * 2 * b->n, st));
  gcm_status s = launch_fields(b, st);
  if (s) return s;
  BatchMeshParams p = mesh_params(b, nullptr, nullptr, 0, nullptr, cnt);
  GCM_CUDA(ctx, launch_batch_mesh(false, b->plan.threads, p, b->plan.layout, b->plan.blocks_count, st));
  count_launch(ctx, 1);
  std::vector<uint64_t> h(2 * (size_t)b->n);
  GCM_CUDA(ctx, cudaMemcpyAsync(h.data(), b->d_inst, sizeof(uint64_t) * 2 * b->n, cudaMemcpyDeviceToHost, st));
  gcm_counts hc{};
  s = read_counts(ctx, cnt, &hc, st);
  if (h_counts) *h_counts = hc;
  if (h_active) std::memcpy(h_active, h.data(), sizeof(uint64_t) * b->n);
  if (h_verts) std::memcpy(h_verts, h.data() + b->n, sizeof(uint64_t) * b->n);
  return s;
}

gcm_status gcm_batch_mesh_async(gcm_batch* b, float* d_pos, float* d_norm, uint64_t capacity, uint64_t* d_offsets,
                                gcm_counts* d_counts, gcm_stream stream) {
  if (!b) return GCM_ERR_INVALID_ARGUMENT;
  gcm_ctx* ctx = b->ctx;
  if (!d_offsets || !d_counts || (capacity && (!d_pos || !d_norm)))
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_batch_mesh_async: NULL argument");
  if (((reinterpret_cast<uintptr_t>(d_pos) | reinterpret_cast<uintptr_t>(d_norm)) & 15u) != 0)
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "position and normal buffers must be 16-byte aligned");
  return mesh_async(b, d_pos, d_norm, capacity, d_offsets, d_counts, static_cast<cudaStream_t>(stream));
}

gcm_status gcm_batch_mesh_graph(gcm_batch* b, float* d_pos, float* d_norm, uint64_t capacity, uint64_t* d_offsets,
                                gcm_counts* d_counts, gcm_stream stream) {
  if (!b) return GCM_ERR_INVALID_ARGUMENT;
  gcm_ctx* ctx = b->ctx;
  if (!d_offsets || !d_counts || (capacity && (!d_pos || !d_norm)))
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_batch_mesh_graph: NULL argument");
  if (((reinterpret_cast<uintptr_t>(d_pos) | reinterpret_cast<uintptr_t>(d_norm)) & 15u) != 0)
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "position and normal buffers must be 16-byte aligned");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const void* key[5] = {d_pos, d_norm, d_offsets, d_counts, stream};
  if (!b->exec || std::memcmp(key, b->g_key, sizeof(key)) != 0 || b->g_cap != capacity) {
    drop_graph(b);
    // capture on a private stream so the caller's stream may be the legacy one
    cudaStream_t cap_st;
    GCM_CUDA(ctx, cudaStreamCreateWithFlags(&cap_st, cudaStreamNonBlocking));
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(cap_st, cudaStreamCaptureModeThreadLocal);
    gcm_status s = GCM_OK;
    if (e == cudaSuccess) {
      s = mesh_async(b, d_pos, d_norm, capacity, d_offsets, d_counts, cap_st);
      e = cudaStreamEndCapture(cap_st, &graph);
    }
    if (e == cudaSuccess && !s) e = cudaGraphInstantiate(&b->exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    cudaStreamDestroy(cap_st);
    if (s) return s;
    if (e != cudaSuccess) return cuda_fail(ctx, e, "graph capture of the batch");
    std::memcpy(b->g_key, key, sizeof(key));
    b->g_cap = capacity;
  }
  GCM_CUDA(ctx, cudaGraphLaunch(b->exec, st));
  count_launch(ctx, 2 + b->blend_ids.size() * 2);
  return GCM_OK;
}

gcm_status gcm_batch_tune(gcm_batch* b, float* d_pos, float* d_norm, uint64_t capacity, const char* cache_path,
                          int* h_threads, uint32_t* h_tile_voxels, gcm_stream stream) {
  if (!b) return GCM_ERR_INVALID_ARGUMENT;
  gcm_ctx* ctx = b->ctx;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const std::string sig = signature(b);
  int best_t = 0;
  uint32_t best_v = 0;
  float best_ms = 0;
  if (!cache_lookup(cache_path, sig, &best_t, &best_v)) {
    uint64_t* d_off = nullptr;
    gcm_counts* d_cnt = nullptr;
    GCM_CUDA(ctx, cudaMalloc(&d_off, sizeof(uint64_t) * (b->n + 1)));
    cudaError_t e = cudaMalloc(&d_cnt, sizeof(gcm_counts));
    cudaEvent_t e0, e1;
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    gcm_status s = e == cudaSuccess ? GCM_OK : cuda_fail(ctx, e, "tuner setup");
    for (int threads : {128, 256}) {
      for (uint32_t vox : {1024u, 2048u, 4096u, 8192u}) {
        if (s) break;
        s = make_plan(b, threads, vox);
        if (s == GCM_ERR_NOT_SUPPORTED) {
          s = GCM_OK;
          continue;
        }
        for (int rep = 0; rep < 2 && !s; ++rep) s = mesh_async(b, d_pos, d_norm, capacity, d_off, d_cnt, st);
        if (s) break;
        cudaEventRecord(e0, st);
        for (int rep = 0; rep < 3 && !s; ++rep) s = mesh_async(b, d_pos, d_norm, capacity, d_off, d_cnt, st);
        cudaEventRecord(e1, st);
        if (cudaEventSynchronize(e1) != cudaSuccess) s = fail(ctx, GCM_ERR_CUDA, "tuner timing failed");
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        ms /= 3;
        gcm_counts hc{};
        if (!s) s = read_counts(ctx, d_cnt, &hc, st);
        if (s == GCM_ERR_OUTPUT_OVERFLOW) s = GCM_OK;  // timing only
        if (!s && (best_t == 0 || ms < best_ms)) {
          best_t = threads;
          best_v = vox;
          best_ms = ms;
        }
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d_off);
    cudaFree(d_cnt);
    if (s) return s;
    if (cache_path) {
      FILE* f = std::fopen(cache_path, "a");
      if (f) {
        std::fprintf(f, "gcm-tune-v1 %s %d %u %.4f\n", sig.c_str(), best_t, best_v, best_ms);
        std::fclose(f);
      }
    }
  }
  gcm_status s = make_plan(b, best_t, best_v);
  if (s) return s;
  if (h_threads) *h_threads = best_t;
  if (h_tile_voxels) *h_tile_voxels = best_v;
  return GCM_OK;
}

gcm_status gcm_ctx_set_launch_shape(gcm_ctx* ctx, int threads, uint32_t tile_voxels) {
  if (!ctx) return GCM_ERR_INVALID_ARGUMENT;
  if (!mesh_threads_supported(threads) || tile_voxels < 64 || tile_voxels > (1u << 20))
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "unsupported launch shape (%d threads, %u voxels)", threads,
                tile_voxels);
  ctx->mesh_threads = threads;
  ctx->tile_voxels = tile_voxels;
  ctx->shape_set = true;
  return GCM_OK;
}

}  // extern "C"
