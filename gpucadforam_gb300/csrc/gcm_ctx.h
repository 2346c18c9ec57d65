// Context object behind the opaque gcm_ctx handle, and the host helpers the
// C-ABI translation units share.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <string>

#include "../../include/gcm.h"
#include "gcm_kernels.h"

constexpr uint64_t kDefaultWaitNs = 2000000000ull;

struct gcm_ctx {
  int device = 0;
  int sm_count = 0;
  size_t smem_optin = 0;
  uint64_t wait_ns = kDefaultWaitNs;
  // fused-kernel launch shape (the autotuner may change both)
  int mesh_threads = GCM_MESH_THREADS;
  uint32_t tile_voxels = GCM_MESH_TILE_VOXELS;
  bool shape_set = false;  // the caller chose the launch shape (else per-form defaults)
  bool prim_exact = false; // primitive fields in the reference's powf arithmetic
  int mesh_path = GCM_MESH_PATH_AUTO;
  std::atomic<uint64_t> launches{0};
  std::string last_error;
  // scratch (device): counts + counters + tile states
  void* scratch = nullptr;
  size_t scratch_bytes = 0;
  // derived field buffer for gcm_mesh_lattice / gcm_mesh_csg
  float* field_buf = nullptr;
  size_t field_bytes = 0;
  float* blend_buf = nullptr;
  size_t blend_bytes = 0;
  // scratch and blend buffer lent by an owner for one request (the server
  // lends ranges of its device pool): never grown or freed by the context; a
  // call that needs more fails with GCM_ERR_OUT_OF_MEMORY
  bool lent = false;
  // pinned host staging for count readback
  gcm_counts* h_pinned = nullptr;
  // .obj welding buffers (grown on demand)
  void* weld_buf = nullptr;
  size_t weld_bytes = 0;
};


namespace gcm {

gcm_status fail(gcm_ctx* ctx, gcm_status s, const char* fmt, ...);
gcm_status cuda_fail(gcm_ctx* ctx, cudaError_t e, const char* what);
gcm_status ensure_scratch(gcm_ctx* ctx, size_t bytes);
gcm_status ensure_buffer(gcm_ctx* ctx, float** buf, size_t* have, size_t bytes);
gcm_status read_counts(gcm_ctx* ctx, const gcm_counts* d, gcm_counts* h, cudaStream_t st);
void count_launch(gcm_ctx* ctx, uint64_t n);
uint32_t grid_blocks(gcm_ctx* ctx, uint64_t work, uint32_t threads, uint32_t per_sm = 8);
// Scratch bytes one plain extraction of `grid` takes (gcm_count_field, then
// gcm_mesh_field[_async] on the fused or the sparse path); 0 for a bad grid.
size_t extraction_scratch_bytes(gcm_ctx* ctx, const gcm_grid* grid, bool sparse);

}  // namespace gcm

#define GCM_CUDA(ctx, call)                                       \
  do {                                                            \
    cudaError_t e_ = (call);                                      \
    if (e_ != cudaSuccess) return gcm::cuda_fail(ctx, e_, #call); \
  } while (0)
