// Runs the reference's own .obj writer (File_output::file_write_obj,
// src/File_output.cu:5-81, compiled from the reference sources by
// oracle/ref/build_ref.py) on a vertex buffer read from a file, on the host.
// The writer copies its input with cudaMemcpy(..., cudaMemcpyDeviceToHost);
// this program links a host-memory stand-in for that one call, so the
// reference's code runs unchanged on a machine without a GPU.
// Test infrastructure only.  Use: obj_ref_writer <pos.f32> <out.obj>
#include <cuda_runtime_api.h>

#include <cstdio>
#include <cstring>
#include <vector>

#include "File_output.h"

extern "C" cudaError_t cudaMemcpy(void* dst, const void* src, size_t count, enum cudaMemcpyKind) {
  std::memcpy(dst, src, count);
  return cudaSuccess;
}

int main(int argc, char** argv) {
  if (argc != 3) return 2;
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 1;
  std::fseek(f, 0, SEEK_END);
  const long bytes = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  std::vector<float4> pos((size_t)bytes / sizeof(float4));
  if (!pos.empty() && std::fread(pos.data(), sizeof(float4), pos.size(), f) != pos.size()) return 1;
  std::fclose(f);
  File_output out;
  out.file_write_obj(pos.data(), (unsigned)pos.size(), argv[2]);
  return 0;
}
