// Times the reference's own scan step: ThrustScanWrapper_lattice
// (src/MarchingCubes_kernel.cu:3198-3203) calls
// thrust::exclusive_scan(device_ptr<uint>(input), device_ptr<uint>(input + n),
// device_ptr<uint>(output)) on the per-voxel vertex counts and occupancy
// (src/Isosurface.cu:425-431).  The same call on n seeded counts in [0, 15],
// timed with CUDA events.  Measurement infrastructure only.
//
//   ref_scan N REPS   ->   prints "N median_ms"
#include <cuda_runtime.h>
#include <thrust/device_ptr.h>
#include <thrust/scan.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <vector>

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: ref_scan N REPS\n");
    return 2;
  }
  const size_t n = std::strtoull(argv[1], nullptr, 10);
  const int reps = std::atoi(argv[2]);
  std::vector<unsigned int> h(n);
  unsigned long long s = 0x9E3779B97F4A7C15ull;
  for (size_t i = 0; i < n; ++i) {
    s = s * 6364136223846793005ull + 1442695040888963407ull;
    h[i] = (unsigned int)(s >> 60);  // 0..15, like vertex counts
  }
  unsigned int *in = nullptr, *out = nullptr;
  if (cudaMalloc(&in, n * 4) != cudaSuccess || cudaMalloc(&out, n * 4) != cudaSuccess) return 3;
  cudaMemcpy(in, h.data(), n * 4, cudaMemcpyHostToDevice);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  std::vector<float> ms;
  for (int r = 0; r < reps + 2; ++r) {
    cudaEventRecord(e0);
    thrust::exclusive_scan(thrust::device_ptr<unsigned int>(in), thrust::device_ptr<unsigned int>(in + n),
                           thrust::device_ptr<unsigned int>(out));
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float t = 0;
    cudaEventElapsedTime(&t, e0, e1);
    if (r >= 2) ms.push_back(t);  // two warm-up calls (first-use allocation of thrust's scratch)
  }
  if (cudaGetLastError() != cudaSuccess) return 4;
  std::sort(ms.begin(), ms.end());
  std::printf("%zu %.6f\n", n, ms[ms.size() / 2]);
  cudaFree(in);
  cudaFree(out);
  return 0;
}
