// Marching-cubes kernels for sm_103a.
//
// mc_mesh_kernel: one pass over the field.  The voxel grid is cut into tiles of
// R consecutive voxel rows of one z-plane, numbered in voxel order, so each
// tile's output is one contiguous run of the reference's vertex buffer.
// Persistent CTAs take tiles in increasing order from an atomic counter; per
// tile a CTA
//   1. stages the (R+1) sample rows of planes z and z+1 in shared memory with
//      bulk (TMA) copies,
//   2. classifies its voxels in warp windows of 32 consecutive voxels of a row,
//   3. scans the window triangle counts,
//   4. gets its output offset through a decoupled look-back over tile states,
//   5. emits triangles with one lane per triangle, so a warp writes one
//      contiguous span of positions and one of normals.
// Output positions and normals are exactly those of the reference
// (classifyVoxel_new + thrust scans + compactVoxels + generate, see
// src/Isosurface.cu:401-572).
#include <cuda_runtime.h>
#include <stdint.h>

#include "gcm_device.cuh"
#include "gcm_kernels.h"

namespace gcm {

namespace {

constexpr int kMapPerWarp = 32 * 5;  // up to 5 triangles for each of 32 voxels

// Register cap per CTA size: resident CTAs per SM the kernel is compiled for.
#ifndef GCM_MESH_MIN_BLOCKS
#define GCM_MESH_MIN_BLOCKS 5
#endif
constexpr int mesh_min_blocks(int threads) { return threads >= 256 ? GCM_MESH_MIN_BLOCKS : 2 * GCM_MESH_MIN_BLOCKS; }

__host__ __device__ inline uint32_t align16(uint32_t x) { return (x + 15u) & ~15u; }

// Staging of one run of `count` floats starting at global element `start`:
// element start + i lands at dst[(start & 3) + i], which keeps source and
// destination equally aligned modulo 16 bytes.  With bulk copies the 16-byte
// aligned middle of the run goes through one cp.async.bulk; the ragged ends
// (at most 3 floats each) and, without bulk copies, the whole run go through
// ordinary loads.
struct Run {
  uint32_t m, head, body;  // alignment shift, leading scalar elements, bulk elements
};

__device__ __forceinline__ Run plan_run(uint64_t start, uint32_t count, bool bulk) {
  Run r;
  r.m = (uint32_t)(start & 3u);
  if (!bulk) {
    r.head = count;
    r.body = 0;
    return r;
  }
  const uint32_t head = (4u - r.m) & 3u;
  r.head = head < count ? head : count;
  r.body = ((count - r.head) / 4u) * 4u;
  return r;
}

__device__ __forceinline__ void stage_scalar(float* dst, const float* __restrict__ src, uint64_t start,
                                             uint32_t count, const Run& r) {
  float* d = dst + r.m;
  const float* s = src + start;
  for (uint32_t i = threadIdx.x; i < r.head; i += blockDim.x) d[i] = __ldg(s + i);
  for (uint32_t i = r.head + r.body + threadIdx.x; i < count; i += blockDim.x) d[i] = __ldg(s + i);
}

__device__ __forceinline__ void stage_bulk(float* dst, const float* __restrict__ src, uint64_t start, const Run& r,
                                           uint64_t* bar) {
  if (r.body) bulk_copy_g2s(dst + r.m + r.head, src + start + r.head, r.body * 4u, bar);
}

// One tile, resolved: rows y0..y0+rows-1 of voxel plane z of a grid.
struct TileGeom {
  const float* f;
  const float* g;
  uint32_t nx, ny, z, y0, rows, bulk;
  Frame fr;
  float iso, lo, hi;
};

// What a tile leaves for the kernel around it (shared memory).
struct TileOut {
  uint64_t prefix;  // first vertex of the tile (emit pass)
  uint32_t tris;    // triangles in the tile
  uint32_t active;  // active voxels in the tile
  uint32_t ok;
};

struct EmitTarget {
  float4* pos;
  float4* norm;
  uint64_t capacity;
  uint64_t* tile_status;
  uint32_t* status;
  uint64_t wait_ns;
};

// Steps 1-5 of one tile (see the file comment).  Every thread of the CTA calls
// it; it ends with a barrier.  Returns false when the CTA has to stop taking
// tiles (a bulk copy did not land within the wait limit).
template <bool BAND, bool EMIT, int THREADS>
__device__ __forceinline__ bool mesh_tile(const TileGeom& tg, uint64_t t, const MeshLayout& L, unsigned char* smem,
                                          uint32_t& parity, const EmitTarget& out, TileOut& res) {
  constexpr uint32_t kWarps = THREADS / 32;
  const uint64_t* s_tri = reinterpret_cast<const uint64_t*>(smem);
  float* s_f0 = reinterpret_cast<float*>(smem + L.f_off);
  float* s_f1 = s_f0 + L.plane_stride;
  float* s_g0 = reinterpret_cast<float*>(smem + L.g_off);
  float* s_g1 = s_g0 + L.plane_stride;
  uint8_t* s_cube = smem + L.cube_off;
  uint32_t* s_win = reinterpret_cast<uint32_t*>(smem + L.win_off);
  uint8_t* s_map = smem + L.map_off;
  uint64_t* s_bar = reinterpret_cast<uint64_t*>(smem + L.bar_off);

  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  const uint32_t nx = tg.nx, vx = nx - 1;
  const uint32_t nwx = (vx + 31u) / 32u;
  const uint32_t rows = tg.rows, z = tg.z, y0 = tg.y0;

  // 1. stage sample rows y0..y0+rows of planes z and z+1
  const uint64_t st0 = ((uint64_t)z * tg.ny + y0) * nx;
  const uint64_t st1 = st0 + (uint64_t)tg.ny * nx;
  const uint32_t cnt = (rows + 1) * nx;
  const bool bulk = tg.bulk != 0;
  const Run r0 = plan_run(st0, cnt, bulk), r1 = plan_run(st1, cnt, bulk);
  if (bulk && tid == 0) {
    // The barrier before this tile ordered every thread's reads of the previous
    // one; the proxy fence orders them before the async-proxy writes.  Expect
    // the bytes first, then issue the copies.
    fence_proxy_async();
    const uint32_t bytes = (r0.body + r1.body) * 4u * (BAND ? 2u : 1u);
    mbar_arrive_expect_tx(s_bar, bytes);
    stage_bulk(s_f0, tg.f, st0, r0, s_bar);
    stage_bulk(s_f1, tg.f, st1, r1, s_bar);
    if (BAND) {
      stage_bulk(s_g0, tg.g, st0, r0, s_bar);
      stage_bulk(s_g1, tg.g, st1, r1, s_bar);
    }
  }
  stage_scalar(s_f0, tg.f, st0, cnt, r0);
  stage_scalar(s_f1, tg.f, st1, cnt, r1);
  if (BAND) {
    stage_scalar(s_g0, tg.g, st0, cnt, r0);
    stage_scalar(s_g1, tg.g, st1, cnt, r1);
  }
  bool lost = false;
  if (bulk) {
    if (!mbar_wait_bounded(s_bar, parity, out.wait_ns)) {
      set_status(out.status, kStatusTimeout);
      res.ok = 0;
      // The copy is still owed to this barrier: wait for it once more before
      // the buffer is reused; if it still has not landed, stop taking tiles.
      lost = !mbar_wait_bounded(s_bar, parity, out.wait_ns);
    }
    parity ^= 1u;
  }
  if (__syncthreads_or(lost)) return false;
  const uint32_t m0 = (uint32_t)(st0 & 3u), m1 = (uint32_t)(st1 & 3u);

  // 2. classify in warp windows of 32 consecutive voxels of a row
  const uint32_t nwin = rows * nwx;
  uint32_t my_active = 0;
  for (uint32_t w = warp; w < nwin; w += kWarps) {
    const uint32_t r = w / nwx, x = (w % nwx) * 32u + lane;
    uint32_t nt = 0;
    if (x < vx) {
      const float* a = s_f0 + m0 + r * nx + x;
      const float* b = s_f1 + m1 + r * nx + x;
      const float c[8] = {a[0], a[1], a[nx + 1], a[nx], b[0], b[1], b[nx + 1], b[nx]};
      const uint32_t ci = cube_index8(c, tg.iso);
      s_cube[r * vx + x] = (uint8_t)ci;
      nt = row_ntris(s_tri[ci]);
    }
    my_active += __popc(__ballot_sync(0xffffffffu, nt > 0));
    const uint32_t wsum = warp_sum_u32(nt);
    if (lane == 0) s_win[w] = wsum;
  }
  if (lane == 0 && my_active) atomicAdd(&res.active, my_active);
  __syncthreads();

  // 3. exclusive scan of the window triangle counts (warp 0)
  if (warp == 0) {
    uint32_t carry = 0;
    for (uint32_t b = 0; b < nwin; b += 32u) {
      const uint32_t v = (b + lane < nwin) ? s_win[b + lane] : 0u;
      const uint32_t inc = warp_incl_scan(v);
      if (b + lane < nwin) s_win[b + lane] = carry + inc - v;
      carry += __shfl_sync(0xffffffffu, inc, 31);
    }
    if (lane == 0) res.tris = carry;
  }
  __syncthreads();
  if (!EMIT) return true;
  const uint64_t tile_verts = 3ull * res.tris;

  // 4. decoupled look-back for the tile's first vertex
  if (warp == 0) {
    const uint64_t excl = lookback_exclusive(out.tile_status, t, tile_verts, out.wait_ns, out.status);
    if (lane == 0) res.prefix = excl;
  }
  __syncthreads();
  if (!res.ok) {
    __syncthreads();
    return true;
  }
  const uint64_t prefix = res.prefix;

  // 5. emit, one lane per triangle
  uint8_t* map = s_map + warp * kMapPerWarp;
  bool dropped = false;
  for (uint32_t w = warp; w < nwin; w += kWarps) {
    const uint32_t r = w / nwx, xb = (w % nwx) * 32u, x = xb + lane;
    uint32_t ci = 0, nt = 0;
    if (x < vx) {
      ci = s_cube[r * vx + x];
      nt = row_ntris(s_tri[ci]);
    }
    const uint32_t inc = warp_incl_scan(nt);
    const uint32_t exc = inc - nt;
    const uint32_t wtot = __shfl_sync(0xffffffffu, inc, 31);
    if (wtot == 0) continue;
    for (uint32_t k = 0; k < nt; ++k) map[exc + k] = (uint8_t)lane;
    __syncwarp();
    const uint64_t wbase = prefix + 3ull * s_win[w];
    for (uint32_t k0 = 0; k0 < wtot; k0 += 32u) {
      const uint32_t k = k0 + lane;
      const uint32_t src = (k < wtot) ? map[k] : 0u;
      const uint32_t sci = __shfl_sync(0xffffffffu, ci, src);
      const uint32_t sexc = __shfl_sync(0xffffffffu, exc, src);
      if (k < wtot) {
        const uint32_t j = k - sexc;  // triangle within its voxel
        const uint32_t sx = xb + src;
        const uint32_t g[3] = {sx, y0 + r, z};
        // corner k of voxel (sx, r) in the staged planes
        const float* f0p = s_f0 + m0 + r * nx + sx;
        const float* f1p = s_f1 + m1 + r * nx + sx;
        auto fval = [&](int kk) { return (corner_z(kk) ? f1p : f0p)[corner_y(kk) * nx + corner_x(kk)]; };
        const uint64_t row = s_tri[sci];
        float3 v[3];
        if (BAND) {
          const float* g0p = s_g0 + m0 + r * nx + sx;
          const float* g1p = s_g1 + m1 + r * nx + sx;
          auto gval = [&](int kk) { return (corner_z(kk) ? g1p : g0p)[corner_y(kk) * nx + corner_x(kk)]; };
#pragma unroll
          for (int mI = 0; mI < 3; ++mI)
            v[mI] = edge_point_band(g, tg.fr, tri_edge_dev(row, 3u * j + mI), fval, gval, tg.lo, tg.hi);
        } else {
#pragma unroll
          for (int mI = 0; mI < 3; ++mI) v[mI] = edge_point_plain(g, tg.fr, tri_edge_dev(row, 3u * j + mI), fval, tg.iso);
        }
        const float3 n = normal_of(v[0], v[1], v[2]);
        const uint64_t idx = wbase + 3ull * k;
        if (idx + 3 <= out.capacity) {
          float4* P = out.pos + idx;
          float4* N = out.norm + idx;
          __stcs(P + 0, make_float4(v[0].x, v[0].y, v[0].z, 1.0f));
          __stcs(P + 1, make_float4(v[1].x, v[1].y, v[1].z, 1.0f));
          __stcs(P + 2, make_float4(v[2].x, v[2].y, v[2].z, 1.0f));
          const float4 nn = make_float4(n.x, n.y, n.z, 0.0f);
          __stcs(N + 0, nn);
          __stcs(N + 1, nn);
          __stcs(N + 2, nn);
        } else {
          dropped = true;
        }
      }
    }
    __syncwarp();
  }
  if (dropped) set_status(out.status, kStatusOverflow);
  __syncthreads();
  return true;
}

__device__ __forceinline__ void mesh_cta_init(unsigned char* smem, const MeshLayout& L) {
  load_tri_table(reinterpret_cast<uint64_t*>(smem));
  if (threadIdx.x == 0) {
    mbar_init(reinterpret_cast<uint64_t*>(smem + L.bar_off), 1);
    fence_mbar_init();
  }
  __syncthreads();
}

}  // namespace

MeshLayout mesh_layout(uint32_t plane_floats, uint32_t tile_voxels, uint32_t windows, bool band, int threads) {
  MeshLayout L;
  const uint32_t plane_bytes = align16(plane_floats * 4);
  L.plane_stride = plane_bytes / 4;
  L.f_off = 2048;  // after the 256-entry triangle table
  L.g_off = L.f_off + 2 * plane_bytes;
  L.cube_off = L.g_off + (band ? 2 * plane_bytes : 0);
  L.win_off = L.cube_off + align16(tile_voxels);
  L.map_off = L.win_off + align16(windows * 4);
  L.bar_off = L.map_off + align16((uint32_t)(threads / 32) * kMapPerWarp);
  L.total = L.bar_off + 16;
  return L;
}

MeshLayout mesh_layout_for(uint32_t nx, uint32_t rows, bool band, int threads) {
  return mesh_layout((rows + 1) * nx + 4, rows * (nx - 1), rows * ((nx - 1 + 31) / 32), band, threads);
}

size_t mesh_smem_bytes(uint32_t nx, uint32_t rows, bool band) { return mesh_layout_for(nx, rows, band, 256).total; }

template <bool BAND, bool EMIT, int THREADS>
__global__ void __launch_bounds__(THREADS, mesh_min_blocks(THREADS)) mc_mesh_kernel(MeshParams p, MeshLayout L) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ uint32_t sh_tile;
  __shared__ TileOut res;
  mesh_cta_init(smem, L);
  const EmitTarget out{p.pos, p.norm, p.capacity, p.tile_status, p.status, p.wait_ns};
  uint32_t parity = 0;
  while (true) {
    if (threadIdx.x == 0) {
      sh_tile = atomicAdd(p.counter, 1u);
      res.tris = 0;
      res.active = 0;
      res.ok = 1;
    }
    __syncthreads();
    const uint32_t t = sh_tile;
    if ((uint64_t)t >= p.ntiles) break;
    TileGeom tg;
    tg.f = p.f;
    tg.g = p.g;
    tg.nx = p.nx;
    tg.ny = p.ny;
    tg.z = t / p.tiles_per_plane;
    tg.y0 = (t % p.tiles_per_plane) * p.rows;
    tg.rows = min(p.rows, p.ny - 1 - tg.y0);
    tg.bulk = p.bulk;
    tg.fr = Frame{{p.vs[0], p.vs[1], p.vs[2]}, {p.gc[0], p.gc[1], p.gc[2]}};
    tg.iso = p.iso;
    tg.lo = p.lo;
    tg.hi = p.hi;
    if (!mesh_tile<BAND, EMIT, THREADS>(tg, t, L, smem, parity, out, res)) break;
    if (threadIdx.x == 0) {
      auto* cnt = p.counts_dev;
      atomicAdd(reinterpret_cast<unsigned long long*>(&cnt->active_voxels), (unsigned long long)res.active);
      if (!EMIT) atomicAdd(reinterpret_cast<unsigned long long*>(&cnt->total_verts), 3ull * res.tris);
      else if ((uint64_t)t == p.ntiles - 1) cnt->total_verts = res.prefix + 3ull * res.tris;
    }
  }
}

// Batch of grids in one launch: the tiles of all instances form one sequence
// (instance by instance, each in its voxel order) and one look-back chain, so
// instance i's vertices start where instance i-1's end.
template <bool EMIT, int THREADS>
__global__ void __launch_bounds__(THREADS, mesh_min_blocks(THREADS)) mc_batch_kernel(BatchMeshParams p, MeshLayout L) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ uint32_t sh_tile;
  __shared__ TileOut res;
  mesh_cta_init(smem, L);
  const EmitTarget out{p.pos, p.norm, p.capacity, p.tile_status, p.status, p.wait_ns};
  uint32_t parity = 0;
  while (true) {
    if (threadIdx.x == 0) {
      sh_tile = atomicAdd(p.counter, 1u);
      res.tris = 0;
      res.active = 0;
      res.ok = 1;
    }
    __syncthreads();
    const uint32_t t = sh_tile;
    if ((uint64_t)t >= p.ntiles) break;
    // instance owning tile t: last i with tile_begin[i] <= t
    uint32_t lo = 0, hi = p.n_inst - 1;
    while (lo < hi) {
      const uint32_t mid = (lo + hi + 1) / 2;
      if (p.inst[mid].tile_begin <= t) lo = mid;
      else hi = mid - 1;
    }
    const BatchInstance& I = p.inst[lo];
    const uint32_t local = t - (uint32_t)I.tile_begin;
    TileGeom tg;
    tg.f = I.f;
    tg.g = I.f;
    tg.nx = I.nx;
    tg.ny = I.ny;
    tg.z = local / I.tiles_per_plane;
    tg.y0 = (local % I.tiles_per_plane) * I.rows;
    tg.rows = min(I.rows, I.ny - 1 - tg.y0);
    tg.bulk = I.bulk;
    tg.fr = Frame{{I.vs[0], I.vs[1], I.vs[2]}, {I.gc[0], I.gc[1], I.gc[2]}};
    tg.iso = I.iso;
    tg.lo = 0.0f;
    tg.hi = 0.0f;
    if (!mesh_tile<false, EMIT, THREADS>(tg, t, L, smem, parity, out, res)) break;
    if (threadIdx.x == 0) {
      auto* cnt = p.counts_dev;
      atomicAdd(reinterpret_cast<unsigned long long*>(&p.inst_active[lo]), (unsigned long long)res.active);
      atomicAdd(reinterpret_cast<unsigned long long*>(&cnt->active_voxels), (unsigned long long)res.active);
      if (!EMIT) {
        atomicAdd(reinterpret_cast<unsigned long long*>(&p.inst_verts[lo]), 3ull * res.tris);
        atomicAdd(reinterpret_cast<unsigned long long*>(&cnt->total_verts), 3ull * res.tris);
      } else {
        if (local == 0) p.offsets[lo] = res.prefix;
        if ((uint64_t)t == p.ntiles - 1) {
          p.offsets[p.n_inst] = res.prefix + 3ull * res.tris;
          cnt->total_verts = res.prefix + 3ull * res.tris;
        }
      }
    }
  }
}

// ----------------------------------------------------------------------------
// Staged reference-form kernels.
// ----------------------------------------------------------------------------

__device__ __forceinline__ void voxel_xyz(uint64_t v, uint32_t nx, uint32_t ny, uint32_t g[3]) {
  const uint64_t mx = nx - 1, mxy = mx * (ny - 1);
  g[2] = (uint32_t)(v / mxy);
  const uint64_t rem = v - (uint64_t)g[2] * mxy;
  g[1] = (uint32_t)(rem / mx);
  g[0] = (uint32_t)(rem - (uint64_t)g[1] * mx);
}

__device__ __forceinline__ void corners_global(const float* __restrict__ f, const uint32_t g[3], uint32_t nx,
                                               uint32_t ny, float c[8]) {
  const uint64_t b = (uint64_t)g[0] + (uint64_t)nx * ((uint64_t)g[1] + (uint64_t)ny * g[2]);
  const uint64_t sy = nx, sz = (uint64_t)nx * ny;
  c[0] = __ldg(f + b);
  c[1] = __ldg(f + b + 1);
  c[2] = __ldg(f + b + sy + 1);
  c[3] = __ldg(f + b + sy);
  c[4] = __ldg(f + b + sz);
  c[5] = __ldg(f + b + sz + 1);
  c[6] = __ldg(f + b + sz + sy + 1);
  c[7] = __ldg(f + b + sz + sy);
}

__global__ void __launch_bounds__(256) mc_classify_kernel(const float* __restrict__ f, uint32_t nx, uint32_t ny,
                                                          uint64_t nvox, float iso, uint32_t* verts, uint32_t* occ,
                                                          uint8_t* cube) {
  __shared__ uint64_t s_tri[256];
  load_tri_table(s_tri);
  __syncthreads();
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < nvox; v += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t g[3];
    voxel_xyz(v, nx, ny, g);
    float c[8];
    corners_global(f, g, nx, ny, c);
    const uint32_t ci = cube_index8(c, iso);
    const uint32_t n = row_nverts(s_tri[ci]);
    if (verts) verts[v] = n;
    if (occ) occ[v] = n > 0;
    if (cube) cube[v] = (uint8_t)ci;
  }
}

__global__ void __launch_bounds__(256) mc_compact_kernel(const uint32_t* __restrict__ occ,
                                                         const uint32_t* __restrict__ scan, uint64_t n,
                                                         uint32_t* out) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    if (occ[i]) out[scan[i]] = (uint32_t)i;
}

template <bool BAND>
__global__ void __launch_bounds__(128) mc_generate_kernel(GenerateParams p) {
  __shared__ uint64_t s_tri[256];
  load_tri_table(s_tri);
  __syncthreads();
  const Frame fr{{p.vs[0], p.vs[1], p.vs[2]}, {p.gc[0], p.gc[1], p.gc[2]}};
  bool dropped = false;
  for (uint64_t a = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; a < p.active;
       a += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t voxel = p.compacted[a];
    uint32_t g[3];
    voxel_xyz(voxel, p.nx, p.ny, g);
    float c[8];
    corners_global(p.f, g, p.nx, p.ny, c);
    const uint32_t ci = cube_index8(c, p.iso);
    const uint64_t row = s_tri[ci];
    const uint32_t nv = row_nverts(row);
    const uint64_t b0 = (uint64_t)g[0] + (uint64_t)p.nx * ((uint64_t)g[1] + (uint64_t)p.ny * g[2]);
    const uint64_t sy = p.nx, sz = (uint64_t)p.nx * p.ny;
    auto off = [&](int k) { return b0 + corner_x(k) + corner_y(k) * sy + corner_z(k) * sz; };
    auto fval = [&](int k) { return __ldg(p.f + off(k)); };
    auto gval = [&](int k) { return __ldg(p.g + off(k)); };
    const uint64_t base = p.verts_scan[voxel];
    for (uint32_t j = 0; j < nv; j += 3) {
      float3 v[3];
      for (int m = 0; m < 3; ++m) {
        const uint32_t e = tri_edge_dev(row, j + m);
        v[m] = BAND ? edge_point_band(g, fr, e, fval, gval, p.lo, p.hi) : edge_point_plain(g, fr, e, fval, p.iso);
      }
      const float3 n = normal_of(v[0], v[1], v[2]);
      const uint64_t idx = base + j;
      if (idx + 3 > p.capacity) {
        dropped = true;
        continue;
      }
      for (int m = 0; m < 3; ++m) {
        p.pos[idx + m] = make_float4(v[m].x, v[m].y, v[m].z, 1.0f);
        p.norm[idx + m] = make_float4(n.x, n.y, n.z, 0.0f);
      }
    }
  }
  if (dropped) set_status(p.status, kStatusOverflow);
}


// ----------------------------------------------------------------------------
// Single-pass exclusive scan of uint32 values (decoupled look-back), 32-bit
// wrap-around output like thrust's scan over uint, 64-bit running total.
// ----------------------------------------------------------------------------
constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;

__global__ void __launch_bounds__(kScanThreads) scan_u32_kernel(ScanParams p) {
  __shared__ uint32_t sh_tile;
  __shared__ uint64_t sh_warp[kScanThreads / 32];
  __shared__ uint64_t sh_prefix;
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  while (true) {
    if (tid == 0) sh_tile = atomicAdd(p.counter, 1u);
    __syncthreads();
    const uint64_t t = sh_tile;
    if (t >= p.ntiles) break;
    const uint64_t base = t * (uint64_t)(kScanThreads * kScanItems) + (uint64_t)tid * kScanItems;
    uint32_t v[kScanItems];
    uint64_t local = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
      v[i] = (base + i < p.n) ? p.in[base + i] : 0u;
      local += v[i];
    }
    // block-exclusive prefix of `local`
    uint64_t inc = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint64_t nb = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= (uint32_t)o) inc += nb;
    }
    if (lane == 31) sh_warp[warp] = inc;
    __syncthreads();
    if (warp == 0) {
      uint64_t wv = lane < (uint32_t)(kScanThreads / 32) ? sh_warp[lane] : 0;
      uint64_t winc = wv;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint64_t nb = __shfl_up_sync(0xffffffffu, winc, o);
        if (lane >= (uint32_t)o) winc += nb;
      }
      const uint64_t tile_total = __shfl_sync(0xffffffffu, winc, 31);
      if (lane < (uint32_t)(kScanThreads / 32)) sh_warp[lane] = winc - wv;
      const uint64_t excl = lookback_exclusive(p.tile_status, t, tile_total, p.wait_ns, p.status);
      if (lane == 0) {
        sh_prefix = excl;
        if (t == p.ntiles - 1 && p.total) *p.total = excl + tile_total;
      }
    }
    __syncthreads();
    uint64_t run = sh_prefix + sh_warp[warp] + (inc - local);
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
      if (base + i < p.n) p.out[base + i] = (uint32_t)run;
      run += v[i];
    }
    __syncthreads();
  }
}

uint32_t scan_tile_elems() { return kScanThreads * kScanItems; }

// ----------------------------------------------------------------------------
// Test kernel for the bounded look-back: one warp per CTA, tiles of aggregate 1,
// tile `stall` never publishes.
// ----------------------------------------------------------------------------
__global__ void __launch_bounds__(32) lookback_stall_kernel(uint32_t ntiles, uint32_t stall, uint64_t wait_ns,
                                                            uint64_t* tile_status, uint32_t* counter,
                                                            uint64_t* prefix_out, uint32_t* status) {
  while (true) {
    uint32_t t = 0;
    if (threadIdx.x == 0) t = atomicAdd(counter, 1u);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= ntiles) break;
    if (t == stall) {
      if (threadIdx.x == 0) prefix_out[t] = ~0ull;
      continue;
    }
    const uint64_t excl = lookback_exclusive(tile_status, t, 1ull, wait_ns, status);
    if (threadIdx.x == 0) prefix_out[t] = excl;
  }
}

// ----------------------------------------------------------------------------
// Launch wrappers.
// ----------------------------------------------------------------------------
namespace {
using MeshFn = void (*)(MeshParams, MeshLayout);
template <int T>
MeshFn mesh_fn_t(bool band, bool emit) {
  if (band) return emit ? mc_mesh_kernel<true, true, T> : mc_mesh_kernel<true, false, T>;
  return emit ? mc_mesh_kernel<false, true, T> : mc_mesh_kernel<false, false, T>;
}
MeshFn mesh_fn(bool band, bool emit, int threads) {
  return threads == 128 ? mesh_fn_t<128>(band, emit) : mesh_fn_t<256>(band, emit);
}
using BatchFn = void (*)(BatchMeshParams, MeshLayout);
BatchFn batch_fn(bool emit, int threads) {
  if (threads == 128) return emit ? mc_batch_kernel<true, 128> : mc_batch_kernel<false, 128>;
  return emit ? mc_batch_kernel<true, 256> : mc_batch_kernel<false, 256>;
}
template <class F>
cudaError_t prepare(F f, size_t smem, int threads, int* blocks_per_sm) {
  cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  // all of the unified L1/shared storage as shared memory: occupancy is
  // limited by shared memory, and the kernel reads global memory only
  // through bulk copies and read-only loads
  e = cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, f, threads, smem);
}
}  // namespace

bool mesh_threads_supported(int threads) { return threads == 128 || threads == 256; }

cudaError_t mesh_prepare(bool band, bool emit, int threads, size_t smem, int* blocks_per_sm) {
  return prepare(mesh_fn(band, emit, threads), smem, threads, blocks_per_sm);
}

cudaError_t launch_mesh(bool band, bool emit, int threads, const MeshParams& p, const MeshLayout& L, uint32_t blocks,
                        cudaStream_t st) {
  mesh_fn(band, emit, threads)<<<blocks, threads, L.total, st>>>(p, L);
  return cudaGetLastError();
}

cudaError_t batch_prepare(bool emit, int threads, size_t smem, int* blocks_per_sm) {
  return prepare(batch_fn(emit, threads), smem, threads, blocks_per_sm);
}

cudaError_t launch_batch_mesh(bool emit, int threads, const BatchMeshParams& p, const MeshLayout& L, uint32_t blocks,
                              cudaStream_t st) {
  batch_fn(emit, threads)<<<blocks, threads, L.total, st>>>(p, L);
  return cudaGetLastError();
}

cudaError_t launch_classify(const float* f, uint32_t nx, uint32_t ny, uint64_t nvox, float iso, uint32_t* verts,
                            uint32_t* occ, uint8_t* cube, uint32_t blocks, cudaStream_t st) {
  mc_classify_kernel<<<blocks, 256, 0, st>>>(f, nx, ny, nvox, iso, verts, occ, cube);
  return cudaGetLastError();
}

cudaError_t launch_compact(const uint32_t* occ, const uint32_t* scan, uint64_t n, uint32_t* out, uint32_t blocks,
                           cudaStream_t st) {
  mc_compact_kernel<<<blocks, 256, 0, st>>>(occ, scan, n, out);
  return cudaGetLastError();
}

cudaError_t launch_generate(bool band, const GenerateParams& p, uint32_t blocks, cudaStream_t st) {
  if (band) mc_generate_kernel<true><<<blocks, 128, 0, st>>>(p);
  else mc_generate_kernel<false><<<blocks, 128, 0, st>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_scan(const ScanParams& p, uint32_t blocks, cudaStream_t st) {
  scan_u32_kernel<<<blocks, kScanThreads, 0, st>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_lookback_stall(uint32_t ntiles, uint32_t stall, uint64_t wait_ns, uint64_t* tile_status,
                                  uint32_t* counter, uint64_t* prefix_out, uint32_t* status, uint32_t blocks,
                                  cudaStream_t st) {
  lookback_stall_kernel<<<blocks, 32, 0, st>>>(ntiles, stall, wait_ns, tile_status, counter, prefix_out, status);
  return cudaGetLastError();
}

}  // namespace gcm
