// Allocation-free variant of the fused marching-cubes extraction.
//
// Some callers cannot allocate device memory at all: code running inside a
// host that owns every allocation itself (an application that sub-allocates
// one pre-reserved arena and forbids cudaMalloc elsewhere), code called while
// a CUDA graph is being captured (cudaMalloc is not capturable), and real-time
// loops where an allocation's implicit synchronisation is not acceptable.
// gcm_mesh_field_noalloc serves them: the caller passes the field, the output
// buffers and a device gcm_counts; the only scratch the kernel needs (its tile
// states and tile counter for the decoupled look-back) lives in the fixed
// array below, which is part of the library's device image.
//
// Limits and rules:
//  * The array is kNoAllocScratchBytes (1 MiB) on every GPU that loads the
//    library, held until the process exits.  It holds the states of at most
//    kNoAllocMaxTiles tiles; tiles are sized up (more voxel rows per tile) to
//    fit, and a grid that still needs more tiles is rejected with
//    GCM_ERR_NOT_SUPPORTED before anything is launched.
//  * All calls share the array and it keeps the previous call's contents;
//    each call clears the part it uses on its stream first.  Calls whose work
//    overlaps on the GPU (different streams, or several host threads) race on
//    the array and produce wrong offsets: serialise them.
//  * The first call on a device resolves the array's device address with
//    cudaGetSymbolAddress (host code may not use the array's name as an
//    address); make that first call before any stream capture.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "../../include/gcm.h"
#include "gcm_kernels.h"

constexpr size_t kNoAllocScratchBytes = 1u << 20;

// The fixed scratch: device code could name it directly; host code only ever
// passes the address cudaGetSymbolAddress returns for the current device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {

constexpr size_t kHeaderBytes = 128;  // [64, 128): tile counter
constexpr uint64_t kNoAllocMaxTiles = (kNoAllocScratchBytes - kHeaderBytes) / sizeof(uint64_t);
constexpr uint32_t kTargetVoxelsPerTile = GCM_MESH_TILE_VOXELS;
constexpr size_t kSmemBudget = 96 * 1024;
constexpr int kMaxDevices = 64;
constexpr int kThreads = GCM_MESH_THREADS;

std::mutex g_setup_mutex;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device (set-up on first use).
cudaError_t scratch_address(int dev, void** out) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return cudaSuccess;
}

}  // namespace

extern "C" gcm_status gcm_mesh_field_noalloc(const float* d_field, const gcm_grid* grid, float iso, float* d_pos,
                                             float* d_norm, uint64_t capacity_verts, gcm_counts* d_counts,
                                             gcm_stream stream) {
  if (!d_field || !grid || !d_counts || (capacity_verts && (!d_pos || !d_norm))) return GCM_ERR_INVALID_ARGUMENT;
  if (((reinterpret_cast<uintptr_t>(d_pos) | reinterpret_cast<uintptr_t>(d_norm)) & 15u) != 0)
    return GCM_ERR_INVALID_ARGUMENT;
  if (grid->nx < 2 || grid->ny < 2 || grid->nz < 2) return GCM_ERR_INVALID_ARGUMENT;
  if (grid->nx > 16384 || grid->ny > 65536 || grid->nz > 65536) return GCM_ERR_NOT_SUPPORTED;

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return GCM_ERR_CUDA;
  int sms = 0, optin = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
    return GCM_ERR_CUDA;

  // Tile shape: whole voxel rows, about GCM_MESH_TILE_VOXELS (1024) voxels,
  // grown until the tile states fit the fixed array, within the shared-memory
  // budget (cubes up to 907^3 fit; 908^3 needs more tiles than the array holds).
  const uint32_t vx = grid->nx - 1, vy = grid->ny - 1, vz = grid->nz - 1;
  const size_t budget = std::min(kSmemBudget, (size_t)optin);
  uint32_t rows =
      std::min<uint32_t>(std::min<uint32_t>(std::max<uint32_t>(1, (kTargetVoxelsPerTile + vx / 2) / vx), vy),
                         gcm::max_tile_rows(vx));
  auto tiles_for = [&](uint32_t r) { return (uint64_t)((vy + r - 1) / r) * vz; };
  while (tiles_for(rows) > kNoAllocMaxTiles && rows < vy && rows < gcm::max_tile_rows(vx) &&
         gcm::mesh_layout_for(grid->nx, rows + 1, gcm::kMeshPlain, kThreads).total <= budget)
    ++rows;
  while (rows > 1 && gcm::mesh_layout_for(grid->nx, rows, gcm::kMeshPlain, kThreads).total > budget) --rows;
  const gcm::MeshLayout layout = gcm::mesh_layout_for(grid->nx, rows, gcm::kMeshPlain, kThreads);
  const size_t smem = layout.total;
  const uint64_t ntiles = tiles_for(rows);
  if (ntiles > kNoAllocMaxTiles || smem > (size_t)optin) return GCM_ERR_NOT_SUPPORTED;

  void* base = nullptr;
  if (scratch_address(dev, &base) != cudaSuccess) return GCM_ERR_CUDA;
  char* b = static_cast<char*>(base);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t used = kHeaderBytes + ntiles * sizeof(uint64_t);
  if (cudaMemsetAsync(b, 0, used, st) != cudaSuccess) return GCM_ERR_CUDA;
  if (cudaMemsetAsync(d_counts, 0, sizeof(gcm_counts), st) != cudaSuccess) return GCM_ERR_CUDA;

  gcm::MeshParams p{};
  p.f = d_field;
  p.g = d_field;
  p.nx = grid->nx;
  p.ny = grid->ny;
  p.nz = grid->nz;
  p.rows = rows;
  p.tiles_per_plane = (vy + rows - 1) / rows;
  p.ntiles = ntiles;
  p.bulk = (reinterpret_cast<uintptr_t>(d_field) & 15u) == 0;
  for (int a = 0; a < 3; ++a) {
    p.vs[a] = grid->voxel_size[a];
    p.gc[a] = grid->grid_center[a];
  }
  p.iso = iso;
  p.pos = reinterpret_cast<float4*>(d_pos);
  p.norm = reinterpret_cast<float4*>(d_norm);
  p.capacity = capacity_verts;
  p.tile_status = reinterpret_cast<uint64_t*>(b + kHeaderBytes);
  p.counter = reinterpret_cast<uint32_t*>(b + 64);
  p.counts_dev = d_counts;
  p.status = &d_counts->status;
  p.wait_ns = 2000000000ull;

  int per_sm = 0;
  if (gcm::mesh_prepare(gcm::kMeshPlain, true, kThreads, smem, &per_sm) != cudaSuccess) return GCM_ERR_CUDA;
  const uint32_t blocks = (uint32_t)std::min<uint64_t>((uint64_t)sms * (uint64_t)std::max(per_sm, 1), ntiles);
  if (gcm::launch_mesh(gcm::kMeshPlain, true, kThreads, p, layout, blocks, st) != cudaSuccess) return GCM_ERR_CUDA;
  return GCM_OK;
}
