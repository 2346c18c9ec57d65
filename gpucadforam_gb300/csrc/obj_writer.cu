// .obj export: File_output::file_write_obj (src/File_output.cu:5-81) on the GPU.
//
// The reference copies every vertex to the host and welds them one by one
// through std::map (O(V log V) on one core).  Here the weld runs on the device
// with the same result:
//   1. each position is quantised as the reference does, coordinate by
//      coordinate: float(int(x * 1000) * 0.001) (float product, truncation,
//      double product, rounding to float);
//   2. a hash table keyed by the quantised coordinates keeps, per distinct
//      position, the smallest vertex number; a vertex is a new .obj vertex
//      when it is that first occurrence, and .obj vertex numbers (1-based)
//      follow first occurrences in vertex order;
//   3. faces with a repeated vertex number are dropped, and of identical
//      ordered faces only the first is kept (second hash table keyed by the
//      triple, entries verified against the face itself);
//   4. faces are emitted as (a, c, b), the reference's swapped winding.
// The host formats the text like the reference's std::ostream output
// ("%g" numbers) in parallel and writes the file.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <string>
#include <thread>
#include <vector>

#include "../../include/gcm.h"
#include "gcm_ctx.h"
#include "gcm_device.cuh"
#include "gcm_kernels.h"

namespace gcm {
namespace {

constexpr uint64_t kEmptyKey = ~0ull;
constexpr uint32_t kEmptyVal = 0xFFFFFFFFu;
constexpr int32_t kKeyLimit = 1 << 20;  // |int(x*1000)| below 2^20: |x| < 1048.576

__device__ __forceinline__ float quantise(float x, int32_t* iq) {
  const int32_t i = __float2int_rz(__fmul_rn(x, 1000.0f));
  *iq = i;
  return __double2float_rn(__dmul_rn((double)i, 0.001));
}

__device__ __forceinline__ uint64_t mix64(uint64_t k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ull;
  k ^= k >> 33;
  return k;
}

struct WeldParams {
  const float4* pos;
  uint64_t n;            // vertices
  uint64_t* keys;        // table_size
  uint32_t* vals;        // table_size
  uint64_t table_mask;
  uint32_t* slot_of;     // n
  float* qxyz;           // 3n quantised coordinates
  uint32_t* status;
};

// Distinct quantised positions -> smallest vertex number.  Quantised integers
// within +-2^20 pack into 63 bits; inside that range the integer triple and the
// float triple the reference keys its std::map on determine each other.
__global__ void __launch_bounds__(256) weld_insert_kernel(WeldParams p) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < p.n; i += (uint64_t)gridDim.x * blockDim.x) {
    const float4 v = p.pos[i];
    int32_t ix, iy, iz;
    const float qx = quantise(v.x, &ix), qy = quantise(v.y, &iy), qz = quantise(v.z, &iz);
    p.qxyz[3 * i + 0] = qx;
    p.qxyz[3 * i + 1] = qy;
    p.qxyz[3 * i + 2] = qz;
    if (ix <= -kKeyLimit || ix >= kKeyLimit || iy <= -kKeyLimit || iy >= kKeyLimit || iz <= -kKeyLimit ||
        iz >= kKeyLimit) {
      set_status(p.status, GCM_ERR_NOT_SUPPORTED);
      p.slot_of[i] = 0;
      continue;
    }
    const uint64_t key = ((uint64_t)(uint32_t)(ix + kKeyLimit) << 42) | ((uint64_t)(uint32_t)(iy + kKeyLimit) << 21) |
                         (uint64_t)(uint32_t)(iz + kKeyLimit);
    uint64_t h = mix64(key) & p.table_mask;
    for (uint64_t probe = 0; probe <= p.table_mask; ++probe) {
      const unsigned long long prev =
          atomicCAS(reinterpret_cast<unsigned long long*>(&p.keys[h]), (unsigned long long)kEmptyKey,
                    (unsigned long long)key);
      if (prev == kEmptyKey || prev == key) {
        atomicMin(&p.vals[h], (uint32_t)i);
        p.slot_of[i] = (uint32_t)h;
        break;
      }
      h = (h + 1) & p.table_mask;
    }
  }
}

__global__ void __launch_bounds__(256) weld_first_kernel(const uint32_t* slot_of, const uint32_t* vals, uint64_t n,
                                                         uint32_t* rep, uint32_t* first) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t r = vals[slot_of[i]];
    rep[i] = r;
    first[i] = (r == (uint32_t)i) ? 1u : 0u;
  }
}

// .obj numbers per vertex (1-based), and the distinct positions in order.
__global__ void __launch_bounds__(256) weld_number_kernel(const uint32_t* rep, const uint32_t* first,
                                                          const uint32_t* first_scan, const float* qxyz, uint64_t n,
                                                          uint32_t* vid, float* out_v, uint64_t cap_v) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    vid[i] = first_scan[rep[i]] + 1u;
    if (first[i] && out_v) {
      const uint64_t k = first_scan[i];
      if (k < cap_v) {
        out_v[3 * k + 0] = qxyz[3 * i + 0];
        out_v[3 * k + 1] = qxyz[3 * i + 1];
        out_v[3 * k + 2] = qxyz[3 * i + 2];
      }
    }
  }
}

__device__ __forceinline__ uint64_t face_hash(uint32_t a, uint32_t b, uint32_t c) {
  return mix64(((uint64_t)a << 32) ^ ((uint64_t)b << 16) ^ (uint64_t)c ^ ((uint64_t)c << 48));
}

// Faces: non-degenerate ones go into a table of face numbers keyed by the
// ordered triple; the smallest face number of each triple survives.
__global__ void __launch_bounds__(256) face_insert_kernel(const uint32_t* vid, uint64_t nf, uint32_t* ftable,
                                                          uint64_t fmask, uint32_t* fslot) {
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < nf; t += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t a = vid[3 * t], b = vid[3 * t + 1], c = vid[3 * t + 2];
    if (a == b || a == c || b == c) {
      fslot[t] = kEmptyVal;
      continue;
    }
    uint64_t h = face_hash(a, b, c) & fmask;
    for (uint64_t probe = 0; probe <= fmask; ++probe) {
      uint32_t cur = atomicCAS(&ftable[h], kEmptyVal, (uint32_t)t);
      if (cur == kEmptyVal) {
        fslot[t] = (uint32_t)h;
        break;
      }
      if (vid[3 * (uint64_t)cur] == a && vid[3 * (uint64_t)cur + 1] == b && vid[3 * (uint64_t)cur + 2] == c) {
        atomicMin(&ftable[h], (uint32_t)t);
        fslot[t] = (uint32_t)h;
        break;
      }
      h = (h + 1) & fmask;
    }
  }
}

__global__ void __launch_bounds__(256) face_keep_kernel(const uint32_t* fslot, const uint32_t* ftable, uint64_t nf,
                                                        uint32_t* keep) {
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < nf; t += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t s = fslot[t];
    keep[t] = (s != kEmptyVal && ftable[s] == (uint32_t)t) ? 1u : 0u;
  }
}

__global__ void __launch_bounds__(256) face_out_kernel(const uint32_t* vid, const uint32_t* keep,
                                                       const uint32_t* keep_scan, uint64_t nf, uint32_t* out_f,
                                                       uint64_t cap_f) {
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < nf; t += (uint64_t)gridDim.x * blockDim.x) {
    if (!keep[t]) continue;
    const uint64_t k = keep_scan[t];
    if (k >= cap_f) continue;
    out_f[3 * k + 0] = vid[3 * t];
    out_f[3 * k + 1] = vid[3 * t + 2];
    out_f[3 * k + 2] = vid[3 * t + 1];
  }
}

uint64_t next_pow2(uint64_t x) {
  uint64_t p = 1024;
  while (p < x) p <<= 1;
  return p;
}

struct WeldLayout {
  uint64_t T, TF;  // table sizes
  size_t off_status, off_keys, off_vals, off_slot, off_q, off_rep, off_first, off_fscan, off_vid, off_ftab, off_fslot, off_keep,
      off_kscan, total;
};

WeldLayout weld_layout(uint64_t n) {
  WeldLayout L;
  const uint64_t nf = n / 3;
  L.T = next_pow2(2 * std::max<uint64_t>(n, 1));
  L.TF = next_pow2(2 * std::max<uint64_t>(nf, 1));
  size_t o = 0;
  auto take = [&](size_t bytes) {
    const size_t at = o;
    o += (bytes + 255) / 256 * 256;
    return at;
  };
  L.off_status = take(64);
  L.off_keys = take(L.T * 8);
  L.off_vals = take(L.T * 4);
  L.off_slot = take(n * 4);
  L.off_q = take(n * 12);
  L.off_rep = take(n * 4);
  L.off_first = take(n * 4);
  L.off_fscan = take(n * 4);
  L.off_vid = take(n * 4);
  L.off_ftab = take(L.TF * 4);
  L.off_fslot = take(nf * 4);
  L.off_keep = take(nf * 4);
  L.off_kscan = take(nf * 4);
  L.total = o;
  return L;
}

template <class T>
T* at(void* base, size_t off) {
  return reinterpret_cast<T*>(static_cast<char*>(base) + off);
}

// Runs steps 1-4 on the device.  d_v (3 floats per .obj vertex) and d_f (3
// uint32 per face, already in (a, c, b) order) may be null to count only.
gcm_status weld(gcm_ctx* ctx, const float* d_pos, uint64_t n, float* d_v, uint64_t cap_v, uint32_t* d_f,
                uint64_t cap_f, uint64_t* nv_out, uint64_t* nf_out, cudaStream_t st) {
  if (n % 3 != 0) return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "vertex count %llu is not a multiple of 3",
                              (unsigned long long)n);
  if (n >= (1ull << 32) - 1) return fail(ctx, GCM_ERR_NOT_SUPPORTED, "more than 2^32 vertices");
  if ((reinterpret_cast<uintptr_t>(d_pos) & 15u) != 0)
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "positions must be 16-byte aligned");
  const uint64_t nf = n / 3;
  const WeldLayout L = weld_layout(n);
  if (L.total > ctx->weld_bytes) {
    if (ctx->weld_buf) cudaFree(ctx->weld_buf);
    ctx->weld_buf = nullptr;
    ctx->weld_bytes = 0;
    GCM_CUDA(ctx, cudaMalloc(&ctx->weld_buf, L.total));
    ctx->weld_bytes = L.total;
  }
  void* B = ctx->weld_buf;
  uint32_t* wstatus = at<uint32_t>(B, L.off_status);
  gcm_status s = GCM_OK;
  GCM_CUDA(ctx, cudaMemsetAsync(wstatus, 0, 64, st));
  GCM_CUDA(ctx, cudaMemsetAsync(at<char>(B, L.off_keys), 0xFF, L.T * 8, st));
  GCM_CUDA(ctx, cudaMemsetAsync(at<char>(B, L.off_vals), 0xFF, L.T * 4, st));
  GCM_CUDA(ctx, cudaMemsetAsync(at<char>(B, L.off_ftab), 0xFF, L.TF * 4, st));
  WeldParams p{};
  p.pos = reinterpret_cast<const float4*>(d_pos);
  p.n = n;
  p.keys = at<uint64_t>(B, L.off_keys);
  p.vals = at<uint32_t>(B, L.off_vals);
  p.table_mask = L.T - 1;
  p.slot_of = at<uint32_t>(B, L.off_slot);
  p.qxyz = at<float>(B, L.off_q);
  p.status = wstatus;
  const uint32_t gb = grid_blocks(ctx, n, 256);
  if (n) {
    weld_insert_kernel<<<gb, 256, 0, st>>>(p);
    GCM_CUDA(ctx, cudaGetLastError());
    weld_first_kernel<<<gb, 256, 0, st>>>(p.slot_of, p.vals, n, at<uint32_t>(B, L.off_rep),
                                         at<uint32_t>(B, L.off_first));
    GCM_CUDA(ctx, cudaGetLastError());
    count_launch(ctx, 2);
  }
  uint64_t nv = 0;
  s = gcm_scan_exclusive_u32(ctx, at<uint32_t>(B, L.off_first), at<uint32_t>(B, L.off_fscan), n, &nv, st);
  if (s) return s;
  uint32_t hstatus = 0;
  GCM_CUDA(ctx, cudaMemcpyAsync(&hstatus, wstatus, 4, cudaMemcpyDeviceToHost, st));
  GCM_CUDA(ctx, cudaStreamSynchronize(st));
  if (hstatus == GCM_ERR_NOT_SUPPORTED)
    return fail(ctx, GCM_ERR_NOT_SUPPORTED, "a coordinate reaches |x| >= 1048.576, beyond the weld key range");
  if (hstatus) return fail(ctx, (gcm_status)hstatus, "weld failed on the device");
  if (n) {
    weld_number_kernel<<<gb, 256, 0, st>>>(at<uint32_t>(B, L.off_rep), at<uint32_t>(B, L.off_first),
                                          at<uint32_t>(B, L.off_fscan), p.qxyz, n, at<uint32_t>(B, L.off_vid), d_v,
                                          cap_v);
    GCM_CUDA(ctx, cudaGetLastError());
    const uint32_t fb = grid_blocks(ctx, nf, 256);
    face_insert_kernel<<<fb, 256, 0, st>>>(at<uint32_t>(B, L.off_vid), nf, at<uint32_t>(B, L.off_ftab), L.TF - 1,
                                          at<uint32_t>(B, L.off_fslot));
    GCM_CUDA(ctx, cudaGetLastError());
    face_keep_kernel<<<fb, 256, 0, st>>>(at<uint32_t>(B, L.off_fslot), at<uint32_t>(B, L.off_ftab), nf,
                                        at<uint32_t>(B, L.off_keep));
    GCM_CUDA(ctx, cudaGetLastError());
    count_launch(ctx, 3);
  }
  uint64_t nk = 0;
  s = gcm_scan_exclusive_u32(ctx, at<uint32_t>(B, L.off_keep), at<uint32_t>(B, L.off_kscan), nf, &nk, st);
  if (s) return s;
  if (nf && d_f) {
    face_out_kernel<<<grid_blocks(ctx, nf, 256), 256, 0, st>>>(at<uint32_t>(B, L.off_vid), at<uint32_t>(B, L.off_keep),
                                                             at<uint32_t>(B, L.off_kscan), nf, d_f, cap_f);
    GCM_CUDA(ctx, cudaGetLastError());
    count_launch(ctx, 1);
  }
  *nv_out = nv;
  *nf_out = nk;
  return GCM_OK;
}

}  // namespace

}  // namespace gcm

namespace {

// "%g" of the float promoted to double: what std::ostream << float prints
// with the default precision (6) and flags.
inline int put_float(char* p, float v) { return std::snprintf(p, 32, "%g", (double)v); }

inline int put_u32(char* p, uint32_t v) {
  char tmp[12];
  int n = 0;
  do {
    tmp[n++] = (char)('0' + v % 10);
    v /= 10;
  } while (v);
  for (int i = 0; i < n; ++i) p[i] = tmp[n - 1 - i];
  return n;
}

// Formats lines [b, e) of either kind into out.
void format_vertices(const float* v, uint64_t b, uint64_t e, std::string& out) {
  out.resize((e - b) * 64);
  char* p = &out[0];
  char* p0 = p;
  for (uint64_t i = b; i < e; ++i) {
    *p++ = 'v';
    *p++ = ' ';
    p += put_float(p, v[3 * i]);
    *p++ = ' ';
    p += put_float(p, v[3 * i + 1]);
    *p++ = ' ';
    p += put_float(p, v[3 * i + 2]);
    *p++ = '\n';
  }
  out.resize((size_t)(p - p0));
}

void format_faces(const uint32_t* f, uint64_t b, uint64_t e, std::string& out) {
  out.resize((e - b) * 40);
  char* p = &out[0];
  char* p0 = p;
  for (uint64_t i = b; i < e; ++i) {
    *p++ = ' ';
    *p++ = 'f';
    *p++ = ' ';
    *p++ = ' ';
    p += put_u32(p, f[3 * i]);
    *p++ = ' ';
    p += put_u32(p, f[3 * i + 1]);
    *p++ = ' ';
    p += put_u32(p, f[3 * i + 2]);
    *p++ = '\n';
  }
  out.resize((size_t)(p - p0));
}

template <class Fmt, class T>
bool write_lines(FILE* fp, const T* data, uint64_t count, Fmt fmt) {
  const unsigned nt = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
  // lines per thread and pass: the count spread over the threads, at least
  // 4096 (thread start-up) and at most 2^20 (64 MB of text per thread buffer)
  const uint64_t block = std::min<uint64_t>(1ull << 20, std::max<uint64_t>(4096, (count + nt - 1) / nt));
  std::vector<std::string> bufs(nt);
  for (uint64_t b0 = 0; b0 < count; b0 += block * nt) {
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; ++t) {
      const uint64_t b = b0 + t * block, e = std::min(count, b + block);
      if (b >= e) {
        bufs[t].clear();
        continue;
      }
      th.emplace_back([&, t, b, e] { fmt(data, b, e, bufs[t]); });
    }
    for (auto& x : th) x.join();
    for (unsigned t = 0; t < nt; ++t)
      if (!bufs[t].empty() && std::fwrite(bufs[t].data(), 1, bufs[t].size(), fp) != bufs[t].size()) return false;
  }
  return true;
}

}  // namespace

using namespace gcm;

extern "C" {

gcm_status gcm_weld_obj(gcm_ctx* ctx, const float* d_pos, uint64_t nverts, float* d_vertices, uint64_t cap_vertices,
                        uint32_t* d_faces, uint64_t cap_faces, uint64_t* h_nvertices, uint64_t* h_nfaces,
                        gcm_stream stream) {
  if (!ctx) return GCM_ERR_INVALID_ARGUMENT;
  if ((!d_pos && nverts) || !h_nvertices || !h_nfaces)
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_weld_obj: NULL argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  uint64_t nv = 0, nf = 0;
  gcm_status s = weld(ctx, d_pos, nverts, d_vertices, cap_vertices, d_faces, cap_faces, &nv, &nf, st);
  if (s) return s;
  GCM_CUDA(ctx, cudaStreamSynchronize(st));
  *h_nvertices = nv;
  *h_nfaces = nf;
  if ((d_vertices && nv > cap_vertices) || (d_faces && nf > cap_faces))
    return fail(ctx, GCM_ERR_OUTPUT_OVERFLOW, "weld output capacity too small");
  return GCM_OK;
}

gcm_status gcm_write_obj(gcm_ctx* ctx, const float* d_pos, uint64_t nverts, const char* path, uint64_t* h_nvertices,
                         uint64_t* h_nfaces, gcm_stream stream) {
  if (!ctx) return GCM_ERR_INVALID_ARGUMENT;
  if ((!d_pos && nverts) || !path) return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_write_obj: NULL argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // count first, then size the outputs exactly
  uint64_t nv = 0, nf = 0;
  gcm_status s = gcm_weld_obj(ctx, d_pos, nverts, nullptr, 0, nullptr, 0, &nv, &nf, stream);
  if (s) return s;
  float* d_v = nullptr;
  uint32_t* d_f = nullptr;
  GCM_CUDA(ctx, cudaMalloc(&d_v, std::max<uint64_t>(nv, 1) * 12));
  cudaError_t e = cudaMalloc(&d_f, std::max<uint64_t>(nf, 1) * 12);
  if (e != cudaSuccess) {
    cudaFree(d_v);
    return cuda_fail(ctx, e, "cudaMalloc(faces)");
  }
  s = gcm_weld_obj(ctx, d_pos, nverts, d_v, nv, d_f, nf, &nv, &nf, stream);
  std::vector<float> hv;
  std::vector<uint32_t> hf;
  if (!s) {
    hv.resize(nv * 3);
    hf.resize(nf * 3);
    e = cudaMemcpyAsync(hv.data(), d_v, nv * 12, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hf.data(), d_f, nf * 12, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) s = cuda_fail(ctx, e, "copy of the welded mesh");
  }
  cudaFree(d_v);
  cudaFree(d_f);
  if (s) return s;
  FILE* fp = std::fopen(path, "wb");
  if (!fp) return fail(ctx, GCM_ERR_IO, "cannot open %s", path);
  bool ok = std::fputs("##Sample latttice new Obj \no Solid \n", fp) >= 0;
  ok = ok && write_lines(fp, hv.data(), nv, format_vertices);
  ok = ok && std::fputs("\n\n", fp) >= 0;
  ok = ok && write_lines(fp, hf.data(), nf, format_faces);
  ok = (std::fclose(fp) == 0) && ok;
  if (!ok) return fail(ctx, GCM_ERR_IO, "write to %s failed", path);
  if (h_nvertices) *h_nvertices = nv;
  if (h_nfaces) *h_nfaces = nf;
  return GCM_OK;
}

}  // extern "C"
