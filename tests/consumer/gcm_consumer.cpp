// A C++ caller of the C ABI, compiled against include/gcm.h and linked to
// libgcm.so the way an application such as the reference's Multitopo would be.
// Test infrastructure (tests/test_abi_consumer.py builds and runs it):
//
//   gcm_consumer layout            sizeof / offsetof of every public struct
//   gcm_consumer reject            argument checks that need no GPU
//   gcm_consumer mesh in.bin out.bin
//                                  gcm_count_field + gcm_mesh_field of a field
//                                  file (nx ny nz uint32, iso, vs[3], gc[3] float,
//                                  then the samples); writes the vertex count
//                                  (uint64) and the positions and normals
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdio>
#include <cstring>
#include <vector>

#include "gcm.h"

#define FIELD(S, F) std::printf("%s %s %zu %zu\n", #S, #F, offsetof(S, F), sizeof(((S*)0)->F))
#define SIZE(S) std::printf("%s sizeof %zu 0\n", #S, sizeof(S))

static int layout() {
  SIZE(gcm_grid); FIELD(gcm_grid, nx); FIELD(gcm_grid, ny); FIELD(gcm_grid, nz); FIELD(gcm_grid, voxel_size);
  FIELD(gcm_grid, grid_center);
  SIZE(gcm_counts); FIELD(gcm_counts, active_voxels); FIELD(gcm_counts, total_verts); FIELD(gcm_counts, status);
  FIELD(gcm_counts, reserved);
  SIZE(gcm_lattice); FIELD(gcm_lattice, mode); FIELD(gcm_lattice, cx); FIELD(gcm_lattice, cy); FIELD(gcm_lattice, cz);
  FIELD(gcm_lattice, d_period); FIELD(gcm_lattice, d_euler); FIELD(gcm_lattice, d_thickness);
  FIELD(gcm_lattice, d_type); FIELD(gcm_lattice, origin);
  SIZE(gcm_primitive); FIELD(gcm_primitive, kind); FIELD(gcm_primitive, op); FIELD(gcm_primitive, flag);
  FIELD(gcm_primitive, reserved); FIELD(gcm_primitive, center); FIELD(gcm_primitive, v3); FIELD(gcm_primitive, p);
  SIZE(gcm_frame); FIELD(gcm_frame, origin); FIELD(gcm_frame, spacing);
  SIZE(gcm_csg_point); FIELD(gcm_csg_point, val); FIELD(gcm_csg_point, t_x); FIELD(gcm_csg_point, t_y);
  FIELD(gcm_csg_point, t_z);
  SIZE(gcm_svl_params); FIELD(gcm_svl_params, nx); FIELD(gcm_svl_params, ny); FIELD(gcm_svl_params, nz);
  FIELD(gcm_svl_params, dx); FIELD(gcm_svl_params, dy); FIELD(gcm_svl_params, dz); FIELD(gcm_svl_params, kind);
  FIELD(gcm_svl_params, period_type); FIELD(gcm_svl_params, period); FIELD(gcm_svl_params, period_x);
  FIELD(gcm_svl_params, period_y); FIELD(gcm_svl_params, period_z); FIELD(gcm_svl_params, lcon);
  FIELD(gcm_svl_params, lcon_1); FIELD(gcm_svl_params, sinewave_z); FIELD(gcm_svl_params, range);
  FIELD(gcm_svl_params, n_coeff); FIELD(gcm_svl_params, max_iter); FIELD(gcm_svl_params, end_res);
  SIZE(gcm_batch_instance); FIELD(gcm_batch_instance, lattice); FIELD(gcm_batch_instance, grid);
  FIELD(gcm_batch_instance, iso); FIELD(gcm_batch_instance, reserved);
  SIZE(gcm_server_config); FIELD(gcm_server_config, device); FIELD(gcm_server_config, lanes);
  FIELD(gcm_server_config, queue_capacity); FIELD(gcm_server_config, fault_flags);
  FIELD(gcm_server_config, device_pool_bytes); FIELD(gcm_server_config, host_pool_bytes);
  FIELD(gcm_server_config, fault_param); FIELD(gcm_server_config, reserved);
  SIZE(gcm_request); FIELD(gcm_request, kind); FIELD(gcm_request, n_prims); FIELD(gcm_request, lattice);
  FIELD(gcm_request, d_prims); FIELD(gcm_request, frame); FIELD(gcm_request, d_field); FIELD(gcm_request, grid);
  FIELD(gcm_request, iso); FIELD(gcm_request, reserved); FIELD(gcm_request, user_tag);
  SIZE(gcm_result); FIELD(gcm_result, ticket); FIELD(gcm_result, user_tag); FIELD(gcm_result, status);
  FIELD(gcm_result, lane); FIELD(gcm_result, total_verts); FIELD(gcm_result, active_voxels); FIELD(gcm_result, pos);
  FIELD(gcm_result, norm); FIELD(gcm_result, on_host); FIELD(gcm_result, reserved); FIELD(gcm_result, t_submit);
  FIELD(gcm_result, t_start); FIELD(gcm_result, t_done);
  SIZE(gcm_server_stats); FIELD(gcm_server_stats, submitted); FIELD(gcm_server_stats, completed);
  FIELD(gcm_server_stats, rejected); FIELD(gcm_server_stats, cancelled); FIELD(gcm_server_stats, failed);
  FIELD(gcm_server_stats, requeued); FIELD(gcm_server_stats, pool_faults); FIELD(gcm_server_stats, device_pool_peak);
  FIELD(gcm_server_stats, device_pool_used); FIELD(gcm_server_stats, host_pool_peak);
  FIELD(gcm_server_stats, lanes_alive); FIELD(gcm_server_stats, pending);
  return 0;
}

static int reject() {
  int bad = 0;
  auto expect = [&](const char* what, gcm_status got, gcm_status want) {
    std::printf("%s %d\n", what, (int)got);
    if (got != want) ++bad;
  };
  expect("ctx_create_null_out", gcm_ctx_create(0, nullptr), GCM_ERR_INVALID_ARGUMENT);
  expect("ctx_destroy_null", gcm_ctx_destroy(nullptr), GCM_OK);
  gcm_grid g{};
  gcm_counts c{};
  expect("mesh_field_null_ctx", gcm_mesh_field(nullptr, nullptr, &g, 0.0f, nullptr, nullptr, 0, &c, nullptr),
         GCM_ERR_INVALID_ARGUMENT);
  expect("count_field_null_ctx", gcm_count_field(nullptr, nullptr, &g, 0.0f, &c, nullptr), GCM_ERR_INVALID_ARGUMENT);
  expect("noalloc_null_field", gcm_mesh_field_noalloc(nullptr, &g, 0.0f, nullptr, nullptr, 0, nullptr, nullptr),
         GCM_ERR_INVALID_ARGUMENT);
  expect("set_mesh_path_null_ctx", gcm_ctx_set_mesh_path(nullptr, GCM_MESH_PATH_SPARSE), GCM_ERR_INVALID_ARGUMENT);
  expect("server_create_null", gcm_server_create(nullptr, nullptr), GCM_ERR_INVALID_ARGUMENT);
  std::printf("abi %d status0 %s\n", gcm_abi_version(), gcm_status_string(GCM_OK));
  return bad;
}

static int mesh(const char* in, const char* out) {
  FILE* f = std::fopen(in, "rb");
  if (!f) return 2;
  uint32_t n[3];
  float hdr[7];
  if (std::fread(n, 4, 3, f) != 3 || std::fread(hdr, 4, 7, f) != 7) return 2;
  const size_t P = (size_t)n[0] * n[1] * n[2];
  std::vector<float> field(P);
  if (std::fread(field.data(), 4, P, f) != P) return 2;
  std::fclose(f);
  gcm_ctx* ctx = nullptr;
  if (gcm_ctx_create(0, &ctx) != GCM_OK) return 3;
  gcm_grid g = {n[0], n[1], n[2], {hdr[1], hdr[2], hdr[3]}, {hdr[4], hdr[5], hdr[6]}};
  float* d_field = nullptr;
  if (cudaMalloc(&d_field, P * 4) != cudaSuccess) return 4;
  cudaMemcpy(d_field, field.data(), P * 4, cudaMemcpyHostToDevice);
  gcm_counts c{};
  if (gcm_count_field(ctx, d_field, &g, hdr[0], &c, nullptr) != GCM_OK) return 5;
  const uint64_t V = c.total_verts;
  float *d_pos = nullptr, *d_norm = nullptr;
  if (cudaMalloc(&d_pos, (V + 1) * 16) != cudaSuccess || cudaMalloc(&d_norm, (V + 1) * 16) != cudaSuccess) return 4;
  gcm_counts c2{};
  if (gcm_mesh_field(ctx, d_field, &g, hdr[0], d_pos, d_norm, V, &c2, nullptr) != GCM_OK) return 6;
  std::vector<float> pos(4 * V), nrm(4 * V);
  cudaMemcpy(pos.data(), d_pos, V * 16, cudaMemcpyDeviceToHost);
  cudaMemcpy(nrm.data(), d_norm, V * 16, cudaMemcpyDeviceToHost);
  FILE* o = std::fopen(out, "wb");
  if (!o) return 2;
  std::fwrite(&V, 8, 1, o);
  std::fwrite(pos.data(), 16, V, o);
  std::fwrite(nrm.data(), 16, V, o);
  std::fclose(o);
  cudaFree(d_field);
  cudaFree(d_pos);
  cudaFree(d_norm);
  gcm_ctx_destroy(ctx);
  return c2.total_verts == V ? 0 : 7;
}

int main(int argc, char** argv) {
  if (argc >= 2 && !std::strcmp(argv[1], "layout")) return layout();
  if (argc >= 2 && !std::strcmp(argv[1], "reject")) return reject();
  if (argc >= 4 && !std::strcmp(argv[1], "mesh")) return mesh(argv[2], argv[3]);
  std::fprintf(stderr, "usage: gcm_consumer layout | reject | mesh in.bin out.bin\n");
  return 2;
}
