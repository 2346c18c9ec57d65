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

#include <algorithm>

#include "gcm_device.cuh"
#include "gcm_kernels.h"

namespace gcm {

namespace {


// Register cap per CTA size: resident CTAs per SM the kernel is compiled for,
// 64 registers for both sizes.  128-thread CTAs: 8, the count the default
// tile's shared memory allows at 512^3 (a cap of 10, 48 registers, spills and
// measured 3% slower there); 256-thread CTAs: 4 (the band form's default
// tiles fit 3 per SM).
#ifndef GCM_MESH_MIN_BLOCKS
#define GCM_MESH_MIN_BLOCKS 4
#endif
constexpr int mesh_min_blocks(int threads) { return threads >= 256 ? GCM_MESH_MIN_BLOCKS : 8; }

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

// One tile, resolved: rows y0..y0+rows-1 of voxel plane z of a grid.  f is
// the classify input (floats, or 4-word accumulator records in the retained
// modes), g the second field (band: normalised field; preview: the fed
// primitive field).
struct TileGeom {
  const float* f;
  const float* g;
  uint32_t nx, ny, z, y0, rows, bulk;
  Frame fr;
  float iso, lo, hi;
  uint32_t op;
  uint32_t inst, local;  // batch bookkeeping: instance and tile within it
};

// What a tile leaves for the kernel around it (shared memory).
struct TileOut {
  uint64_t prefix;  // first vertex of the tile (emit pass)
  uint32_t tris;    // triangles in the tile
  uint32_t active;  // active voxels in the tile
  uint32_t ok;
  uint32_t next_window;  // emission work counter
};

struct EmitTarget {
  float4* pos;
  float4* norm;
  uint64_t capacity;
  uint64_t* tile_status;
  uint32_t* status;
  uint64_t wait_ns;
};

// The staging buffer: planes z and z+1 of the classify input, then (band and
// preview modes) of the second field.
struct Planes {
  float *f0, *f1, *g0, *g1;
};

__device__ __forceinline__ Planes planes_of(unsigned char* smem, const MeshLayout& L) {
  unsigned char* base = smem + L.f_off;
  Planes P;
  P.f0 = reinterpret_cast<float*>(base);
  P.f1 = P.f0 + L.plane_stride;
  P.g0 = P.f1 + L.plane_stride;
  P.g1 = P.g0 + L.plane_stride;
  return P;
}

__device__ __forceinline__ uint64_t* bar_of(unsigned char* smem, const MeshLayout& L) {
  return reinterpret_cast<uint64_t*>(smem + L.bar_off);
}

// Phase 1: issue the staging of tile tg (every thread calls it; thread 0
// issues the bulk copies, every thread loads the ragged ends).  The caller
// guarantees that no thread still reads the buffer.
template <int MODE>
__device__ __forceinline__ void tile_stage(const TileGeom& tg, const MeshLayout& L, unsigned char* smem) {
  constexpr uint32_t W = mode_fw(MODE);
  const Planes P = planes_of(smem, L);
  uint64_t* bar = bar_of(smem, L);
  const uint64_t st0 = ((uint64_t)tg.z * tg.ny + tg.y0) * tg.nx;
  const uint64_t st1 = st0 + (uint64_t)tg.ny * tg.nx;
  const uint32_t cnt = (tg.rows + 1) * tg.nx;
  const bool bulk = tg.bulk != 0;
  // classify input in units of floats (W per sample), second field per sample
  const Run r0 = plan_run(W * st0, W * cnt, bulk), r1 = plan_run(W * st1, W * cnt, bulk);
  const Run q0 = plan_run(st0, cnt, bulk), q1 = plan_run(st1, cnt, bulk);
  if (bulk && threadIdx.x == 0) {
    // Every thread's reads of this buffer were ordered by a barrier before
    // this call; the proxy fence orders them before the async-proxy writes.
    // Expect the bytes first, then issue the copies.
    fence_proxy_async();
    const uint32_t bytes = (r0.body + r1.body + (mode_has_g(MODE) ? q0.body + q1.body : 0u)) * 4u;
    mbar_arrive_expect_tx(bar, bytes);
    stage_bulk(P.f0, tg.f, W * st0, r0, bar);
    stage_bulk(P.f1, tg.f, W * st1, r1, bar);
    if (mode_has_g(MODE)) {
      stage_bulk(P.g0, tg.g, st0, q0, bar);
      stage_bulk(P.g1, tg.g, st1, q1, bar);
    }
  }
  stage_scalar(P.f0, tg.f, W * st0, W * cnt, r0);
  stage_scalar(P.f1, tg.f, W * st1, W * cnt, r1);
  if (mode_has_g(MODE)) {
    stage_scalar(P.g0, tg.g, st0, cnt, q0);
    stage_scalar(P.g1, tg.g, st1, cnt, q1);
  }
}

// Phase 2: wait for the staging (bounded).  Returns false when the CTA has to
// stop taking tiles (a copy did not land within twice the limit).
__device__ __forceinline__ bool tile_wait(const TileGeom& tg, const MeshLayout& L, unsigned char* smem,
                                          uint32_t& parity, const EmitTarget& out, TileOut& res) {
  bool lost = false;
  if (tg.bulk) {
    uint64_t* bar = bar_of(smem, L);
    if (!mbar_wait_bounded(bar, parity, out.wait_ns)) {
      set_status(out.status, kStatusTimeout);
      res.ok = 0;
      // The copy is still owed to this barrier: wait for it once more before
      // the buffer is reused; if it still has not landed, stop taking tiles.
      lost = !mbar_wait_bounded(bar, parity, out.wait_ns);
    }
    parity ^= 1u;
  }
  return !__syncthreads_or(lost);
}

// Window w of a tile as (row, window within the row), stepped without a
// division: windows are taken with a fixed stride per warp.
struct WindowCursor {
  uint32_t r, xw;
  __device__ __forceinline__ WindowCursor(uint32_t w, uint32_t nwx) : r(0), xw(w) { advance(0, nwx); }
  __device__ __forceinline__ void advance(uint32_t by, uint32_t nwx) {
    xw += by;
    while (xw >= nwx) {
      xw -= nwx;
      ++r;
    }
  }
};

// Corner k of a voxel inside the solid: the cube-index bit of each mode.
// Plain and band: f < iso (classifyVoxel_new, src/MarchingCubes_kernel.cu:
// 3207-3249).  Region: the accumulated sign, (float)val < iso.  Preview: the
// accumulated sign combined with the fed field (classifyVoxel,
// src/MarchingCubes_kernel.cu:869-1052): union (val < iso) | (f < iso),
// difference (f >= iso) & (val < iso), intersection (val < iso) & (f < iso).
// Lattice previews (the same kernel with `fixed` or `dynamic` set), with the
// open band lo < L < hi of the lattice field L in g: fixed combines the fed
// primitive field f with the band (difference (f >= iso) & band); dynamic
// combines the accumulated sign with it (difference (val < iso) & (L < lo |
// L > hi), as the reference pairs it).
template <int MODE>
__device__ __forceinline__ bool corner_inside(float fval, float gval, uint32_t op, float iso, float lo, float hi) {
  if (MODE == kMeshPlain || MODE == kMeshBand) return fval < iso;
  if (MODE == kMeshLatFixed) {
    const bool band = (gval > lo) && (gval < hi);
    if (op == GCM_CSG_SUBTRACT) return (fval >= iso) && band;
    if (op == GCM_CSG_INTERSECT) return (fval < iso) && band;
    return (fval < iso) || band;
  }
  const bool a = (float)__float_as_int(fval) < iso;
  if (MODE == kMeshRegion) return a;
  if (MODE == kMeshLatDynamic) {
    if (op == GCM_CSG_SUBTRACT) return a && ((gval < lo) || (gval > hi));
    if (op == GCM_CSG_INTERSECT) return a && (gval > lo) && (gval < hi);
    return a || ((gval > lo) && (gval < hi));
  }
  if (op == GCM_CSG_SUBTRACT) return (gval >= iso) && a;
  if (op == GCM_CSG_INTERSECT) return a && (gval < iso);
  return a || (gval < iso);
}

// Phase 3: classify in warp windows of 32 consecutive voxels of a row, scan the
// window triangle counts and write the tile's edge table.  Ends with a barrier.
template <int MODE, int THREADS>
__device__ __forceinline__ void tile_classify(const TileGeom& tg, const MeshLayout& L, unsigned char* smem,
                                              TileOut& res) {
  constexpr uint32_t kWarps = THREADS / 32;
  constexpr uint32_t W = mode_fw(MODE);
  const uint64_t* s_tri = reinterpret_cast<const uint64_t*>(smem);
  const Planes P = planes_of(smem, L);
  uint8_t* s_cube = smem + L.cube_off;
  uint32_t* s_win = reinterpret_cast<uint32_t*>(smem + L.win_off);
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t nx = tg.nx, vx = nx - 1, nwx = (vx + 31u) / 32u, nwin = tg.rows * nwx;
  const uint64_t st0 = ((uint64_t)tg.z * tg.ny + tg.y0) * nx;
  // shifts of the staged planes: classify input (W floats per sample), second field
  const uint32_t m0 = (uint32_t)((W * st0) & 3u), m1 = (uint32_t)((W * (st0 + (uint64_t)tg.ny * nx)) & 3u);
  const uint32_t n0 = (uint32_t)(st0 & 3u), n1 = (uint32_t)((st0 + (uint64_t)tg.ny * nx) & 3u);
  if (threadIdx.x >= THREADS - 12) {
    // edge table, two words per edge: [first corner's offset : 24][second
    // corner's offset : 24][first bits : 3][second bits : 3], and (retained
    // modes) the byte offset of the first corner's accumulated fraction for
    // the edge's axis.  Offsets are shared-memory bytes from the voxel's
    // first sample (plane z + 1 lies `dplane` floats after plane z) of the
    // field the vertex is interpolated in; they stay below 2^18.  Plain and
    // band edges run edge_a -> edge_b; retained edges run from the corner with
    // the lower coordinate (generateTriangles_lattice_kernel,
    // src/MarchingCubes_kernel.cu:2087-2098).
    const uint32_t e = threadIdx.x - (THREADS - 12);
    const bool retained = mode_lower_edges(MODE);
    const uint32_t dplane = L.plane_stride + (retained ? n1 - n0 : m1 - m0);
    auto off = [&](uint32_t k) {
      return 4u * ((uint32_t)corner_z((int)k) * dplane + (uint32_t)corner_y((int)k) * nx + (uint32_t)corner_x((int)k));
    };
    auto bits = [&](uint32_t k) { return (uint32_t)(corner_x((int)k) | (corner_y((int)k) << 1) | (corner_z((int)k) << 2)); };
    uint32_t ka = (uint32_t)edge_a((int)e), kb = (uint32_t)edge_b((int)e);
    uint64_t word1 = 0;
    if (retained) {
      const uint32_t axis_bit = bits(ka) ^ bits(kb);
      if (bits(ka) & axis_bit) {
        const uint32_t tk = ka;
        ka = kb;
        kb = tk;
      }
      const uint32_t axis = axis_bit == 1u ? 0u : (axis_bit == 2u ? 1u : 2u);
      // record of corner ka in the staged accumulator planes (m0 = m1 = 0),
      // word 1 + axis of it (t_x, t_y, t_z)
      word1 = 4u * ((uint32_t)corner_z((int)ka) * L.plane_stride +
                    4u * ((uint32_t)corner_y((int)ka) * nx + (uint32_t)corner_x((int)ka)) + 1u + axis);
    }
    uint64_t* te = reinterpret_cast<uint64_t*>(smem + L.edge_off) + 2u * e;
    te[0] = (uint64_t)off(ka) | ((uint64_t)off(kb) << 24) | ((uint64_t)bits(ka) << 48) | ((uint64_t)bits(kb) << 51);
    te[1] = word1;
  }
  uint32_t my_active = 0;
  WindowCursor cur(warp, nwx);
  for (uint32_t w = warp; w < nwin; w += kWarps, cur.advance(kWarps, nwx)) {
    const uint32_t r = cur.r, x = cur.xw * 32u + lane;
    uint32_t nt = 0;
    if (x < vx) {
      const float* a = P.f0 + m0 + W * (r * nx + x);
      const float* c1 = P.f1 + m1 + W * (r * nx + x);
      const float c[8] = {a[0], a[W], a[W * (nx + 1)], a[W * nx], c1[0], c1[W], c1[W * (nx + 1)], c1[W * nx]};
      float gv[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      if (MODE == kMeshPreview || MODE == kMeshLatFixed || MODE == kMeshLatDynamic) {
        const float* ga = P.g0 + n0 + r * nx + x;
        const float* gb = P.g1 + n1 + r * nx + x;
        gv[0] = ga[0]; gv[1] = ga[1]; gv[2] = ga[nx + 1]; gv[3] = ga[nx];
        gv[4] = gb[0]; gv[5] = gb[1]; gv[6] = gb[nx + 1]; gv[7] = gb[nx];
      }
      uint32_t ci = 0;
#pragma unroll
      for (int k = 0; k < 8; ++k) ci |= (uint32_t)corner_inside<MODE>(c[k], gv[k], tg.op, tg.iso, tg.lo, tg.hi) << k;
      s_cube[r * vx + x] = (uint8_t)ci;
      nt = (uint32_t)(s_tri[ci] & 0xFu);
    }
    // triangle counts are 0..5: the window's total from three ballots
    const CountPlanes cp = count_planes(nt);
    my_active += __popc(cp.b0 | cp.b1 | cp.b2);
    const uint32_t wsum = planes_total(cp);
    if (lane == 0) s_win[w] = wsum;
  }
  if (lane == 0 && my_active) atomicAdd(&res.active, my_active);
  __syncthreads();
  if (warp == 0) {
    uint32_t carry = 0;
    for (uint32_t bb = 0; bb < nwin; bb += 32u) {
      const uint32_t v = (bb + lane < nwin) ? s_win[bb + lane] : 0u;
      const uint32_t inc = warp_incl_scan(v);
      if (bb + lane < nwin) s_win[bb + lane] = carry + inc - v;
      carry += __shfl_sync(0xffffffffu, inc, 31);
    }
    if (lane == 0) res.tris = carry;
  }
  __syncthreads();
}

// floor(v / d) for v, d < 2^16 as a multiply-high by m = ceil(2^32 / d)
// (exact there: the error term v * (m - 2^32 / d) / 2^32 stays below 1/d);
// d == 1 has no 32-bit multiplier and is passed through.
struct SmallDiv {
  uint32_t d, m;
  __device__ __forceinline__ explicit SmallDiv(uint32_t d_) : d(d_), m(d_ > 1 ? 0xFFFFFFFFu / d_ + 1u : 0u) {}
  __device__ __forceinline__ uint32_t operator()(uint32_t v) const { return d > 1 ? __umulhi(v, m) : v; }
};

// Triangle list entry: the voxel's index within the tile (row * vx + x,
// 16 bits) and the triangle's three edges (12 bits).
__device__ __forceinline__ uint32_t list_entry(uint32_t v, uint32_t e3) { return v | (e3 << 16); }

// Phase 4: decoupled look-back for the tile's first vertex, then emission.
// The tile's triangles are listed in output order (as many as the list holds
// per round) and emitted one lane per triangle in full warps.  Warp 0 walks
// back while the other warps list the first round's triangles, taking windows
// from a shared counter; warp 0 joins when its look-back ends.  Ends with a
// barrier.
template <int MODE, int THREADS>
__device__ __forceinline__ void tile_emit(const TileGeom& tg, uint64_t t, const MeshLayout& L, unsigned char* smem,
                                          const EmitTarget& out, TileOut& res) {
  constexpr uint32_t kWarps = THREADS / 32;
  constexpr bool kRetained = mode_retained_normal(MODE);
  const uint64_t* s_tri = reinterpret_cast<const uint64_t*>(smem);
  const Planes P = planes_of(smem, L);
  const uint8_t* s_cube = smem + L.cube_off;
  const uint32_t* s_win = reinterpret_cast<const uint32_t*>(smem + L.win_off);
  const uint64_t* s_edge = reinterpret_cast<const uint64_t*>(smem + L.edge_off);
  uint32_t* s_list = reinterpret_cast<uint32_t*>(smem + L.list_off);
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  float4* xp = reinterpret_cast<float4*>(smem + L.xpose_off) + warp * 96u;  // this warp's 96 vertices
  // triangle of the chunk's vertex lane + 32k
  const uint32_t q3[3] = {lane / 3u, (lane + 32u) / 3u, (lane + 64u) / 3u};
  const uint32_t nx = tg.nx, vx = nx - 1, nwx = (vx + 31u) / 32u, nwin = tg.rows * nwx;
  const SmallDiv by_vx(vx), by_nwx(nwx);
  const uint64_t st0 = ((uint64_t)tg.z * tg.ny + tg.y0) * nx;
  const uint32_t m0 = (uint32_t)(st0 & 3u);  // shift of single-float planes
  const uint32_t tris = res.tris;
  // list the triangles [base, base + n) of the tile: entry u = triangle base + u
  auto build = [&](uint32_t base, uint32_t n, auto&& next_window) {
    for (uint32_t w = next_window(); w < nwin; w = next_window()) {
      const uint32_t r = by_nwx(w), x = (w - r * nwx) * 32u + lane;
      const uint32_t v = r * vx + x;
      uint64_t row = 0;
      uint32_t nt = 0;
      if (x < vx) {
        row = s_tri[s_cube[v]];
        nt = (uint32_t)(row & 0xFu);
      }
      const uint32_t most = __reduce_max_sync(0xffffffffu, nt);
      if (most == 0) continue;
      const uint32_t first = s_win[w] + planes_excl(count_planes(nt)) - base;  // wraps below base
      // unrolled over the (at most 5) triangles of a voxel, so every edge group
      // is a constant shift; the warp stops after its largest count
#pragma unroll
      for (uint32_t j = 0; j < 5; ++j) {
        if (j >= most) break;
        const uint32_t u = first + j;
        if (j < nt && u < n) s_list[u] = list_entry(v, tri_edges3(row, j));
      }
    }
  };
  auto shared_windows = [&] {
    uint32_t w = 0;
    if (lane == 0) w = atomicAdd(&res.next_window, 1u);
    return __shfl_sync(0xffffffffu, w, 0);
  };
  if (warp == 0) {
    const uint64_t excl = lookback_exclusive(out.tile_status, t, 3ull * tris, out.wait_ns, out.status);
    if (lane == 0) res.prefix = excl;
  }
  const uint32_t n0 = min(L.list_cap, tris);
  if (n0) build(0, n0, shared_windows);
  __syncthreads();
  const bool ok = res.ok != 0;
  const uint64_t prefix = res.prefix;
  if (!ok || tris == 0) {
    __syncthreads();  // every thread has read the record
    return;
  }
  VoxelCorners V;
  axis_corners(tg.z, tg.fr.gc[2], tg.fr.vs[2], V.z0, V.z1);
  // sample (x, r) of plane z: F[r * nx + x] (plain, band; the band's second
  // field 2 planes further), G[r * nx + x] (preview field), accumulator
  // record at A[4 * (r * nx + x)]
  const float* F = P.f0 + m0;
  const float* G = P.g0 + m0;
  const float* A = P.f0;
  const float w_norm = kRetained ? 0.5f : 0.0f;
  bool dropped = false;
  for (uint32_t base = 0; base < tris; base += L.list_cap) {
    const uint32_t n = min(L.list_cap, tris - base);
    if (base) {
      uint32_t next = warp;
      build(base, n, [&] {
        const uint32_t w = next;
        next += kWarps;
        return w;
      });
      __syncthreads();
    }
    for (uint32_t u0 = warp * 32u; u0 < n; u0 += THREADS) {
      // lane = triangle u0 + lane; the chunk's vertices are written in order
      // through shared memory so that every store covers 512 contiguous bytes
      const uint32_t u = u0 + lane;
      const bool live = u < n;
      float3 nrm = make_float3(0.0f, 0.0f, 0.0f);
      if (live) {
        const uint32_t ent = s_list[u];
        const uint32_t v = ent & 0xFFFFu, e3 = ent >> 16;
        const uint32_t r = by_vx(v), x = v - r * vx;
        axis_corners(x, tg.fr.gc[0], tg.fr.vs[0], V.x0, V.x1);
        axis_corners(tg.y0 + r, tg.fr.gc[1], tg.fr.vs[1], V.y0, V.y1);
        const uint32_t s = v + r;  // sample (x, r): r * nx + x
        const char* Fv = reinterpret_cast<const char*>(F + s);
        const char* Gv = reinterpret_cast<const char*>(G + s);
        const char* Av = reinterpret_cast<const char*>(A + 4u * s);
        auto at = [](const char* base, uint32_t off) { return *reinterpret_cast<const float*>(base + off); };
        float3 vtx[3];
#pragma unroll
        for (int m = 0; m < 3; ++m) {
          const uint64_t* te = s_edge + 2u * ((e3 >> (8 - 4 * m)) & 0xFu);
          const uint64_t ed = te[0];
          const uint32_t oa = (uint32_t)ed & 0xFFFFFFu, ob = (uint32_t)(ed >> 24) & 0xFFFFFFu;
          const uint32_t bits = (uint32_t)(ed >> 48), ba = bits & 7u, bb = bits >> 3;
          if (MODE == kMeshBand) {
            const char* Nv = Fv + 8u * L.plane_stride;
            vtx[m] = edge_point_band_v(at(Fv, oa), at(Fv, ob), at(Nv, oa), at(Nv, ob), ba, bb, V, tg.lo, tg.hi);
          } else if (MODE == kMeshRegion) {
            vtx[m] = lerp3(corner_sel(V, ba), corner_sel(V, bb), at(Av, (uint32_t)te[1]));
          } else if (MODE == kMeshPreview) {
            vtx[m] = edge_point_retained(tg.iso, corner_sel(V, ba), corner_sel(V, bb), at(Gv, oa), at(Gv, ob),
                                         at(Av, (uint32_t)te[1]));
          } else if (MODE == kMeshLatFixed) {
            vtx[m] = edge_point_latfixed(tg.iso, tg.lo, tg.hi, corner_sel(V, ba), corner_sel(V, bb), at(Fv, oa),
                                         at(Fv, ob), at(Gv, oa), at(Gv, ob));
          } else if (MODE == kMeshLatDynamic) {
            vtx[m] = edge_point_latdyn(tg.lo, tg.hi, corner_sel(V, ba), corner_sel(V, bb), at(Gv, oa), at(Gv, ob),
                                       at(Av, (uint32_t)te[1]));
          } else {
            vtx[m] = edge_point_plain_v(at(Fv, oa), at(Fv, ob), corner_sel(V, ba), corner_sel(V, bb), tg.iso);
          }
        }
        // the retained modes' generate kernel takes calcNormal(v0, v2, v1) with
        // w = 0.5 (src/MarchingCubes_kernel.cu:2178-2189)
        nrm = kRetained ? normal_of(vtx[0], vtx[2], vtx[1]) : normal_of(vtx[0], vtx[1], vtx[2]);
        xp[3 * lane + 0] = make_float4(vtx[0].x, vtx[0].y, vtx[0].z, 1.0f);
        xp[3 * lane + 1] = make_float4(vtx[1].x, vtx[1].y, vtx[1].z, 1.0f);
        xp[3 * lane + 2] = make_float4(vtx[2].x, vtx[2].y, vtx[2].z, 1.0f);
      }
      const uint32_t nv = 3u * min(32u, n - u0);      // vertices of the chunk
      const uint64_t cb = prefix + 3ull * (base + u0);  // its first output vertex
      float4* gp = out.pos + cb;
      float4* gn = out.norm + cb;
      __syncwarp();
      if (nv == 96u && cb + 96u <= out.capacity) {
        // whole chunk, inside the output
        __stcs(gp + lane, xp[lane]);
        __stcs(gp + lane + 32u, xp[lane + 32u]);
        __stcs(gp + lane + 64u, xp[lane + 64u]);
        __syncwarp();
        xp[lane] = make_float4(nrm.x, nrm.y, nrm.z, w_norm);
        __syncwarp();
        __stcs(gn + lane, xp[q3[0]]);
        __stcs(gn + lane + 32u, xp[q3[1]]);
        __stcs(gn + lane + 64u, xp[q3[2]]);
      } else {
        // ragged or overflowing chunk: a triangle is written only when all of
        // its vertices fit
        if (live && cb + 3ull * lane + 3 > out.capacity) dropped = true;
#pragma unroll
        for (uint32_t k = 0; k < 3; ++k) {
          const uint32_t q = lane + 32u * k;
          if (q < nv && cb + 3ull * q3[k] + 3 <= out.capacity) __stcs(gp + q, xp[q]);
        }
        __syncwarp();
        if (live) xp[lane] = make_float4(nrm.x, nrm.y, nrm.z, w_norm);
        __syncwarp();
#pragma unroll
        for (uint32_t k = 0; k < 3; ++k) {
          const uint32_t q = lane + 32u * k;
          if (q < nv && cb + 3ull * q3[k] + 3 <= out.capacity) __stcs(gn + q, xp[q3[k]]);
        }
      }
      __syncwarp();
    }
    __syncthreads();
  }
  if (dropped) set_status(out.status, kStatusOverflow);
}

__device__ __forceinline__ void mesh_cta_init(unsigned char* smem, const MeshLayout& L) {
  load_tri_table_counted(reinterpret_cast<uint64_t*>(smem));
  if (threadIdx.x == 0) {
    mbar_init(bar_of(smem, L), 1);
    fence_mbar_init();
  }
  __syncthreads();
}

// The tile loop shared by the single-grid and the batch kernel: take a tile,
// stage, classify, look back and emit, repeat.  `geom(t)` resolves tile t,
// `book(tg, t, res)` (thread 0) records a finished tile.  Thread 0 writes the
// tile number and resets the tile record after the barrier that ends the
// previous tile, when no thread reads either any more; every thread reads the
// tile number only after the barrier that follows.
template <int MODE, bool EMIT, int THREADS, class Geom, class Book>
__device__ __forceinline__ void tile_loop(unsigned char* smem, const MeshLayout& L, uint32_t* counter, uint64_t ntiles,
                                          const EmitTarget& out, Geom&& geom, Book&& book) {
  __shared__ uint32_t sh_tile;
  __shared__ TileOut res;
  mesh_cta_init(smem, L);
  uint32_t parity = 0;
  while (true) {
    if (threadIdx.x == 0) {
      sh_tile = atomicAdd(counter, 1u);
      res.tris = 0;
      res.active = 0;
      res.ok = 1;
      res.next_window = 0;
    }
    __syncthreads();
    const uint32_t t = sh_tile;
    if ((uint64_t)t >= ntiles) return;
    const TileGeom tg = geom(t);
    tile_stage<MODE>(tg, L, smem);
    if (!tile_wait(tg, L, smem, parity, out, res)) return;
    tile_classify<MODE, THREADS>(tg, L, smem, res);
    if (EMIT) tile_emit<MODE, THREADS>(tg, t, L, smem, out, res);
    // classify and emit end with a barrier after their last use of the
    // staged planes and of the record: thread 0 may book and reset at once
    if (threadIdx.x == 0) book(tg, t, res);
  }
}

}  // namespace

MeshLayout mesh_layout(uint32_t plane_floats, uint32_t tile_voxels, uint32_t windows, int mode, int threads) {
  MeshLayout L;
  const uint32_t plane_bytes = align16(plane_floats * 4);
  L.plane_stride = plane_bytes / 4;
  // at most 6144 entries: tiles of very wide rows take more rounds instead
  L.list_cap = std::min<uint32_t>(6144, std::max<uint32_t>(64, (GCM_MESH_LIST_PER_2VOX * tile_voxels / 2 + 31) / 32 * 32));
  L.f_off = 2048;  // after the 256-entry triangle table
  L.cube_off = L.f_off + (mode_has_g(mode) ? 4 : 2) * plane_bytes;
  L.win_off = L.cube_off + align16(tile_voxels);
  L.edge_off = L.win_off + align16(windows * 4);
  L.list_off = L.edge_off + 256;  // 12 edges x 2 words
  L.xpose_off = L.list_off + align16(L.list_cap * 4);
  L.bar_off = L.xpose_off + (uint32_t)(threads / 32) * 96u * 16u;
  L.total = L.bar_off + 16;
  return L;
}

MeshLayout mesh_layout_for(uint32_t nx, uint32_t rows, int mode, int threads) {
  return mesh_layout(mode_fw(mode) * (rows + 1) * nx + 4, rows * (nx - 1), rows * ((nx - 1 + 31) / 32), mode,
                     threads);
}

size_t mesh_smem_bytes(uint32_t nx, uint32_t rows, int mode) { return mesh_layout_for(nx, rows, mode, 256).total; }

template <int MODE, bool EMIT, int THREADS>
__global__ void __launch_bounds__(THREADS, mesh_min_blocks(THREADS)) mc_mesh_kernel(MeshParams p, MeshLayout L) {
  extern __shared__ __align__(16) unsigned char smem[];
  const EmitTarget out{p.pos, p.norm, p.capacity, p.tile_status, p.status, p.wait_ns};
  auto geom = [&](uint32_t t) {
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
    tg.op = p.op;
    tg.inst = 0;
    tg.local = t;
    return tg;
  };
  auto book = [&](const TileGeom&, uint32_t t, const TileOut& res) {
    auto* cnt = p.counts_dev;
    atomicAdd(reinterpret_cast<unsigned long long*>(&cnt->active_voxels), (unsigned long long)res.active);
    if (!EMIT) atomicAdd(reinterpret_cast<unsigned long long*>(&cnt->total_verts), 3ull * res.tris);
    else if ((uint64_t)t == p.ntiles - 1) cnt->total_verts = res.prefix + 3ull * res.tris;
  };
  tile_loop<MODE, EMIT, THREADS>(smem, L, p.counter, p.ntiles, out, geom, book);
}

// Batch of grids in one launch: the tiles of all instances form one sequence
// (instance by instance, each in its voxel order) and one look-back chain, so
// instance i's vertices start where instance i-1's end.
template <bool EMIT, int THREADS>
__global__ void __launch_bounds__(THREADS, mesh_min_blocks(THREADS)) mc_batch_kernel(BatchMeshParams p, MeshLayout L) {
  extern __shared__ __align__(16) unsigned char smem[];
  const EmitTarget out{p.pos, p.norm, p.capacity, p.tile_status, p.status, p.wait_ns};
  auto geom = [&](uint32_t t) {
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
    tg.op = 0;
    tg.inst = lo;
    tg.local = local;
    return tg;
  };
  auto book = [&](const TileGeom& tg, uint32_t t, const TileOut& res) {
    auto* cnt = p.counts_dev;
    atomicAdd(reinterpret_cast<unsigned long long*>(&p.inst_active[tg.inst]), (unsigned long long)res.active);
    atomicAdd(reinterpret_cast<unsigned long long*>(&cnt->active_voxels), (unsigned long long)res.active);
    if (!EMIT) {
      atomicAdd(reinterpret_cast<unsigned long long*>(&p.inst_verts[tg.inst]), 3ull * res.tris);
      atomicAdd(reinterpret_cast<unsigned long long*>(&cnt->total_verts), 3ull * res.tris);
    } else {
      if (tg.local == 0) p.offsets[tg.inst] = res.prefix;
      if ((uint64_t)t == p.ntiles - 1) {
        p.offsets[p.n_inst] = res.prefix + 3ull * res.tris;
        cnt->total_verts = res.prefix + 3ull * res.tris;
      }
    }
  };
  tile_loop<kMeshPlain, EMIT, THREADS>(smem, L, p.counter, p.ntiles, out, geom, book);
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
constexpr int kScanRounds = 4;  // 128-element rounds per warp and tile
constexpr uint32_t kScanWarpElems = 32 * 4 * kScanRounds;

namespace {

__device__ __forceinline__ uint64_t warp_inclusive_u64(uint64_t x, uint32_t lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint64_t nb = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (uint32_t)o) x += nb;
  }
  return x;
}

}  // namespace

// Exclusive scan of 32-bit values with 64-bit running sums (the tile prefixes
// and the total are 64-bit; each output is the prefix modulo 2^32, as a
// 32-bit scan's would be).  Tiles of kScanThreads * 16 elements are claimed in
// order from a counter and chained by the decoupled look-back.  Each warp
// scans a contiguous segment of 512 elements in four rounds of 128: lane l
// holds elements 4l .. 4l + 3 of a round (one 16-byte load and store when
// VEC: both arrays 16-byte aligned), so every access is coalesced.
template <bool VEC>
__global__ void __launch_bounds__(kScanThreads, 6) scan_u32_kernel(ScanParams p) {
  __shared__ uint32_t sh_tile;
  __shared__ uint64_t sh_warp[kScanThreads / 32];
  __shared__ uint64_t sh_prefix;
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  while (true) {
    if (tid == 0) sh_tile = atomicAdd(p.counter, 1u);
    __syncthreads();  // also: every warp has read the previous tile's sh_warp and sh_prefix
    const uint64_t t = sh_tile;
    if (t >= p.ntiles) break;
    const uint64_t seg = t * (uint64_t)(kScanThreads / 32 * kScanWarpElems) + (uint64_t)warp * kScanWarpElems;
    uint4 v[kScanRounds];
    uint64_t inc[kScanRounds], warp_total = 0;
#pragma unroll
    for (int k = 0; k < kScanRounds; ++k) {
      const uint64_t i = seg + (uint64_t)k * 128 + 4u * lane;
      if (VEC && i + 3 < p.n) {
        v[k] = __ldcs(reinterpret_cast<const uint4*>(p.in + i));
      } else {
        v[k].x = i < p.n ? p.in[i] : 0u;
        v[k].y = i + 1 < p.n ? p.in[i + 1] : 0u;
        v[k].z = i + 2 < p.n ? p.in[i + 2] : 0u;
        v[k].w = i + 3 < p.n ? p.in[i + 3] : 0u;
      }
      const uint64_t s4 = (uint64_t)v[k].x + v[k].y + v[k].z + v[k].w;
      inc[k] = warp_inclusive_u64(s4, lane);
      warp_total += __shfl_sync(0xffffffffu, inc[k], 31);
    }
    if (lane == 31) sh_warp[warp] = warp_total;
    __syncthreads();
    if (warp == 0) {
      const uint64_t wv = lane < (uint32_t)(kScanThreads / 32) ? sh_warp[lane] : 0;
      const uint64_t winc = warp_inclusive_u64(wv, lane);
      const uint64_t tile_total = __shfl_sync(0xffffffffu, winc, 31);
      if (lane < (uint32_t)(kScanThreads / 32)) sh_warp[lane] = winc - wv;
      const uint64_t excl = lookback_exclusive(p.tile_status, t, tile_total, p.wait_ns, p.status);
      if (lane == 0) {
        sh_prefix = excl;
        if (t == p.ntiles - 1 && p.total) *p.total = excl + tile_total;
      }
    }
    __syncthreads();
    uint64_t run = sh_prefix + sh_warp[warp];
#pragma unroll
    for (int k = 0; k < kScanRounds; ++k) {
      const uint64_t i = seg + (uint64_t)k * 128 + 4u * lane;
      const uint64_t s4 = (uint64_t)v[k].x + v[k].y + v[k].z + v[k].w;
      const uint64_t e = run + inc[k] - s4;
      uint4 o;
      o.x = (uint32_t)e;
      o.y = (uint32_t)(e + v[k].x);
      o.z = (uint32_t)(e + v[k].x + v[k].y);
      o.w = (uint32_t)(e + v[k].x + v[k].y + v[k].z);
      if (VEC && i + 3 < p.n) {
        __stcs(reinterpret_cast<uint4*>(p.out + i), o);
      } else {
        if (i < p.n) p.out[i] = o.x;
        if (i + 1 < p.n) p.out[i + 1] = o.y;
        if (i + 2 < p.n) p.out[i + 2] = o.z;
        if (i + 3 < p.n) p.out[i + 3] = o.w;
      }
      run += __shfl_sync(0xffffffffu, inc[k], 31);
    }
  }
}

uint32_t scan_tile_elems() { return kScanThreads / 32 * kScanWarpElems; }

// ----------------------------------------------------------------------------
// Sparse path: windows of 32 consecutive voxels of a row, in voxel order
// (window (row, wx) holds voxels wx*32 .. wx*32+31 of voxel row row = y + vy*z).
// mc_window_count_kernel: a warp per row at a time, a lane per voxel, corners
// read straight from the field (neighbouring lanes and rows share them through
// L1 and L2); writes each window's triangle count and adds the active voxels
// and vertices to the counts.  mc_window_emit_kernel: after an exclusive scan
// of the window counts, a warp visits only the windows that hold triangles,
// classifies them again and writes each lane's triangles at the window's offset
// plus the lane's prefix: the reference's vertex order, with the same vertex
// arithmetic as every other path.  No look-back and no tile staging, so a
// surface that touches a few percent of the voxels costs little more than one
// read of the field.
// ----------------------------------------------------------------------------
constexpr uint32_t kWinBatch = 4;  // windows a warp handles at once (independent loads in flight)
// A window is 31 voxels of a row: its 32 lanes load 32 consecutive sample
// columns, and lane l's voxel takes column l + 1 from the next lane (lane 31
// only supplies that column).
constexpr uint32_t kWinVox = 31;

static_assert(windows_per_row(62) == 2 && windows_per_row(63) == 3, "windows of kWinVox voxels");

// c[k] for a run-time k without local memory: three levels of selects.
__device__ __forceinline__ float sel8(const float c[8], int k) {
  const float a0 = (k & 1) ? c[1] : c[0], a1 = (k & 1) ? c[3] : c[2], a2 = (k & 1) ? c[5] : c[4],
              a3 = (k & 1) ? c[7] : c[6];
  const float b0 = (k & 2) ? a1 : a0, b1 = (k & 2) ? a3 : a2;
  return (k & 4) ? b1 : b0;
}

// The four samples of column x of the voxel row at rb: (y, z), (y+1, z),
// (y, z+1), (y+1, z+1).
__device__ __forceinline__ float4 load_column(const float* __restrict__ f, uint64_t rb, uint32_t x, uint64_t sy,
                                              uint64_t sz) {
  const float* q = f + rb + x;
  return make_float4(__ldg(q), __ldg(q + sy), __ldg(q + sz), __ldg(q + sy + sz));
}

// Inside bits of a column (bit i: component i < iso, the classify test).
__device__ __forceinline__ uint32_t column_bits(float4 s, float iso) {
  return (uint32_t)(s.x < iso) | ((uint32_t)(s.y < iso) << 1) | ((uint32_t)(s.z < iso) << 2) |
         ((uint32_t)(s.w < iso) << 3);
}

// Cube index from the inside bits of columns x (m) and x + 1 (n): corners
// 0 (x,y,z) 1 (x+1,y,z) 2 (x+1,y+1,z) 3 (x,y+1,z) 4 (x,y,z+1) 5 (x+1,y,z+1)
// 6 (x+1,y+1,z+1) 7 (x,y+1,z+1): the order of cube_index8.  m's bits go to
// corners 0, 3, 4, 7 and n's to 1, 2, 5, 6.
__device__ __forceinline__ uint32_t cube_from_columns(uint32_t m, uint32_t n) {
  return (m & 1u) | ((m & 6u) << 2) | ((m & 8u) << 4) | ((n & 3u) << 1) | ((n & 12u) << 3);
}

// One window batch, classified: each lane's column samples and its voxel's
// cube index per window.
struct WindowBatch {
  float4 col[kWinBatch];
  uint32_t ci[kWinBatch];
};


// One window batch, classified: window k of voxel row rbk[k] (its first
// sample), each lane's column samples and its voxel's cube index (0 for lane
// 31 and past the row's end).
__device__ __forceinline__ void classify_batch(const float* __restrict__ f, const uint64_t* rbk,
                                                    const uint32_t* wx, uint32_t nb, uint32_t vx, uint64_t sy,
                                                    uint64_t sz, float iso, uint32_t lane, WindowBatch& B) {
#pragma unroll
  for (uint32_t k = 0; k < kWinBatch; ++k) {
    B.col[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const uint32_t x = wx[k] * kWinVox + lane;
    if (k < nb && x <= vx) B.col[k] = load_column(f, rbk[k], x, sy, sz);
  }
#pragma unroll
  for (uint32_t k = 0; k < kWinBatch; ++k) {
    const uint32_t x = wx[k] * kWinVox + lane;
    const uint32_t m = column_bits(B.col[k], iso);
    const uint32_t n = __shfl_down_sync(0xffffffffu, m, 1);
    B.ci[k] = (k < nb && lane < kWinVox && x < vx) ? cube_from_columns(m, n) : 0u;
  }
}

// Count pass: a warp task is one window column over up to kCountRows voxel
// rows of one z-plane.  It loads each sample line of planes z and z + 1 once,
// keeps its inside bits, and forms every row's column bits from two adjacent
// lines.  Tasks run window column fastest, so the warps of a wave read one
// contiguous slab of the field.
constexpr uint32_t kCountRows = 8;

template <bool WRITE>
__global__ void __launch_bounds__(256) mc_window_count_kernel(const float* __restrict__ f, uint32_t nx, uint32_t ny,
                                                              uint32_t nz, float iso, uint32_t* __restrict__ win_tris,
                                                              gcm_counts* counts, TileStates tiles) {
  __shared__ uint64_t s_tri[256];
  load_tri_table_counted(s_tri);
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t vx = nx - 1, vy = ny - 1, vz = nz - 1, nwx = windows_per_row(vx);
  const uint32_t nyb = (vy + kCountRows - 1) / kCountRows;
  const uint64_t tasks = (uint64_t)vz * nyb * nwx, sy = nx, sz = (uint64_t)nx * ny;
  const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
  uint32_t active = 0;
  uint64_t tris = 0;
  // task t = wx + nwx * (yb + nyb * z), stepped by `warps` as a mixed-radix
  // counter (no divisions in the loop)
  uint64_t t = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  uint32_t wx = (uint32_t)(t % nwx), yb = (uint32_t)((t / nwx) % nyb);
  uint64_t zz = t / nwx / nyb;
  const uint32_t dwx = (uint32_t)(warps % nwx), dyb = (uint32_t)((warps / nwx) % nyb);
  const uint64_t dz = warps / nwx / nyb;
  for (; t < tasks; t += warps) {
    const uint32_t z = (uint32_t)zz;
    const uint32_t y0 = yb * kCountRows, nr = min(kCountRows, vy - y0);
    const uint32_t x = wx * kWinVox + lane;
    const bool has = x <= vx, voxel = lane < kWinVox && x < vx;
    const float* p0 = f + (uint64_t)y0 * sy + (uint64_t)z * sz + x;
    // With tile states from the field kernel: the task's samples (columns
    // 31 wx .. 31 wx + 31, lines y0 .. y0 + nr, planes z and z + 1) lie in at
    // most 2 x 2 x 2 tiles; if all of them are inside, or all outside, every
    // cube index is 0 or 255 and the samples need not be read.
    bool known = false;
    if (tiles.state) {
      const uint32_t xs = wx * kWinVox, xe = min(xs + kWinVox, vx);
      const uint32_t bx = (lane & 1u) ? xe / GCM_CSG_TILE_X : xs / GCM_CSG_TILE_X;
      const uint32_t by = (lane & 2u) ? (y0 + nr) / GCM_CSG_TILE_Y : y0 / GCM_CSG_TILE_Y;
      const uint32_t bz = (lane & 4u) ? (z + 1) / GCM_CSG_TILE_Z : z / GCM_CSG_TILE_Z;
      const uint32_t st = __ldg(tiles.state + bx + (uint64_t)tiles.tx * (by + (uint64_t)tiles.ty * bz));
      // both collectives run on every lane; only then are their results combined
      const uint32_t st0 = __shfl_sync(0xffffffffu, st, 0);
      const bool same = __all_sync(0xffffffffu, st == st0);
      known = same && st0 != kTileMixed;
    }
    uint32_t line[kCountRows + 1];  // bit 0: plane z, bit 2: plane z + 1
#pragma unroll
    for (uint32_t i = 0; i <= kCountRows; ++i) {
      float a = 0.0f, b = 0.0f;
      if (!known && i <= nr && has) {
        a = __ldg(p0 + i * sy);
        b = __ldg(p0 + i * sy + sz);
      }
      line[i] = (uint32_t)(a < iso) | ((uint32_t)(b < iso) << 2);
    }
    uint32_t nt[kCountRows], task_tris = 0;
    // a task whose lines all lie on one side of the isovalue (every column,
    // both planes) has cube indices 0 or 255 only: no triangles
    uint32_t lor = 0, land = 5u;
#pragma unroll
    for (uint32_t i = 0; i <= kCountRows; ++i) {
      lor |= line[i];
      land &= line[i];
    }
    const bool mixed = !known && __ballot_sync(0xffffffffu, lor != 0u) != 0u &&
                       __ballot_sync(0xffffffffu, land != 5u) != 0u;
#pragma unroll
    for (uint32_t i = 0; i < kCountRows; ++i) nt[i] = 0;
    if (mixed) {
#pragma unroll
      for (uint32_t i = 0; i < kCountRows; ++i) {
        const uint32_t m = line[i] | (line[i + 1] << 1);
        const uint32_t n = __shfl_down_sync(0xffffffffu, m, 1);
        nt[i] = (voxel && i < nr) ? (uint32_t)(s_tri[cube_from_columns(m, n)] & 0xFu) : 0u;
        active += nt[i] > 0;
        task_tris += nt[i];
      }
    }
    tris += task_tris;
    if (WRITE) {
      // the rows' window sums, then lane i stores row i's
      uint32_t mine = 0;
      if (mixed) {
#pragma unroll
        for (uint32_t i = 0; i < kCountRows; ++i) {
          const uint32_t wsum = __reduce_add_sync(0xffffffffu, nt[i]);
          if (lane == i) mine = wsum;
        }
      }
      if (lane < nr) win_tris[((uint64_t)z * vy + y0 + lane) * nwx + wx] = mine;
    }
    wx += dwx;
    uint32_t carry = wx >= nwx;
    if (carry) wx -= nwx;
    yb += dyb + carry;
    carry = yb >= nyb;
    if (carry) yb -= nyb;
    zz += dz + carry;
  }
  const uint64_t wa = warp_sum_u64(active), wt = warp_sum_u64(tris);
  if (lane == 0 && (wa | wt)) {
    atomicAdd(reinterpret_cast<unsigned long long*>(&counts->active_voxels), (unsigned long long)wa);
    atomicAdd(reinterpret_cast<unsigned long long*>(&counts->total_verts), 3ull * wt);
  }
}

// Per warp of the emit kernel: the batch's voxels (corner values, cube
// index, first output triangle) and its triangle list (window, lane and
// triangle number per entry), so that every lane emits one triangle per step.
constexpr uint32_t kEmitWarps = 4;
constexpr uint32_t kEmitList = kWinBatch * 32u * 5u;
struct EmitShared {
  float4 corner[kWinBatch * 32u][2];
  uint64_t first[kWinBatch * 32u];
  uint8_t cube[kWinBatch * 32u];
  uint16_t list[kEmitList];
};

__global__ void __launch_bounds__(kEmitWarps * 32, 8) mc_window_emit_kernel(WindowEmitParams p) {
  __shared__ uint64_t s_tri[256];
  __shared__ EmitShared s_em[kEmitWarps];
  load_tri_table_counted(s_tri);
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31u;
  EmitShared& E = s_em[threadIdx.x >> 5];
  const uint32_t nx = p.nx, ny = p.ny, vx = nx - 1, vy = ny - 1, nwx = windows_per_row(vx);
  const uint64_t rows = (uint64_t)vy * (p.nz - 1), sy = nx, sz = (uint64_t)nx * ny;
  const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
  const Frame fr{{p.vs[0], p.vs[1], p.vs[2]}, {p.gc[0], p.gc[1], p.gc[2]}};
  bool dropped = false;
  // The warp's stream of windows that hold triangles: its voxel rows
  // row = y + vy * z (stepped by `warps` without divisions), in each row the
  // groups of 32 windows, in each group the windows whose count is not zero.
  // A batch takes the next kWinBatch windows of the stream, across rows, so
  // that rows with one or two such windows still fill the emission lanes.
  uint64_t row = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  uint32_t yy = (uint32_t)(row % vy);
  uint64_t zz = row / vy;
  const uint32_t dyy = (uint32_t)(warps % vy);
  const uint64_t dzz = warps / vy;
  uint32_t g0 = 0, todo = 0;  // the current group and its windows not yet taken (warp-uniform)
  auto load_group = [&]() {
    const uint32_t wl = g0 + lane;
    todo = __ballot_sync(0xffffffffu, row < rows && wl < nwx && __ldg(p.win_tris + row * nwx + wl) != 0u);
  };
  auto next_group = [&]() {
    g0 += 32u;
    if (g0 >= nwx) {
      g0 = 0;
      row += warps;
      yy += dyy;
      const uint32_t carry = yy >= vy ? 1u : 0u;
      zz += dzz + carry;
      if (carry) yy -= vy;
    }
    load_group();
  };
  load_group();
  while (true) {
    // the next (up to) kWinBatch windows that hold triangles, all at once
    uint32_t wx[kWinBatch], wy[kWinBatch], wz[kWinBatch];
    uint64_t wrow[kWinBatch];
    uint32_t nb = 0;
#pragma unroll
    for (uint32_t k = 0; k < kWinBatch; ++k) {
      while (todo == 0u && row < rows) next_group();
      wx[k] = 0;
      wy[k] = 0;
      wz[k] = 0;
      wrow[k] = 0;
      if (todo) {
        wx[k] = g0 + (uint32_t)(__ffs(todo) - 1);
        wy[k] = yy;
        wz[k] = (uint32_t)zz;
        wrow[k] = row;
        todo &= todo - 1;
        nb = k + 1;
      }
    }
    if (nb == 0) break;  // the stream is exhausted
    {
        uint64_t off[kWinBatch], rbk[kWinBatch];
#pragma unroll
        for (uint32_t k = 0; k < kWinBatch; ++k) {
          off[k] = k < nb ? __ldg(p.win_off + wrow[k] * nwx + wx[k]) : 0ull;
          rbk[k] = (uint64_t)wy[k] * sy + (uint64_t)wz[k] * sz;
        }
        WindowBatch B;
        classify_batch(p.f, rbk, wx, nb, vx, sy, sz, p.iso, lane, B);
        // list the batch's triangles; stage each active voxel's corners
        __syncwarp();  // the previous batch's entries are read
        uint32_t listed = 0;
#pragma unroll
        for (uint32_t k = 0; k < kWinBatch; ++k) {
          const uint32_t nt = (uint32_t)(s_tri[B.ci[k]] & 0xFu);
          const CountPlanes cp = count_planes(nt);
          const uint32_t excl = planes_excl(cp), slot = k * 32u + lane;
          // the x + 1 column: the next lane's
          float4 n4;
          n4.x = __shfl_down_sync(0xffffffffu, B.col[k].x, 1);
          n4.y = __shfl_down_sync(0xffffffffu, B.col[k].y, 1);
          n4.z = __shfl_down_sync(0xffffffffu, B.col[k].z, 1);
          n4.w = __shfl_down_sync(0xffffffffu, B.col[k].w, 1);
          if (nt) {
            // kCorner order: 0 (x,y,z) 1 (x+1,y,z) 2 (x+1,y+1,z) 3 (x,y+1,z) | 4..7 at z+1
            E.corner[slot][0] = make_float4(B.col[k].x, n4.x, n4.y, B.col[k].y);
            E.corner[slot][1] = make_float4(B.col[k].z, n4.z, n4.w, B.col[k].w);
            E.first[slot] = off[k] + excl;
            E.cube[slot] = (uint8_t)B.ci[k];
            for (uint32_t j = 0; j < nt; ++j) E.list[listed + excl + j] = (uint16_t)((slot << 3) | j);
          }
          listed += planes_total(cp);
        }
        __syncwarp();
        for (uint32_t u = lane; u < listed; u += 32u) {
          const uint32_t ent = E.list[u], slot = ent >> 3, j = ent & 7u;
          const uint32_t k = slot >> 5, l = slot & 31u;
          const float4 ca = E.corner[slot][0], cb = E.corner[slot][1];
          const float c[8] = {ca.x, ca.y, ca.z, ca.w, cb.x, cb.y, cb.z, cb.w};
          const uint64_t tri_row = s_tri[E.cube[slot]];
          uint32_t wxk = wx[0], wyk = wy[0], wzk = wz[0];
#pragma unroll
          for (uint32_t q = 1; q < kWinBatch; ++q) {
            wxk = (k == q) ? wx[q] : wxk;
            wyk = (k == q) ? wy[q] : wyk;
            wzk = (k == q) ? wz[q] : wzk;
          }
          const uint32_t x = wxk * kWinVox + l;
          VoxelCorners V;
          axis_corners(x, fr.gc[0], fr.vs[0], V.x0, V.x1);
          axis_corners(wyk, fr.gc[1], fr.vs[1], V.y0, V.y1);
          axis_corners(wzk, fr.gc[2], fr.vs[2], V.z0, V.z1);
          float3 v[3];
#pragma unroll
          for (int m = 0; m < 3; ++m) {
            const int e = (int)tri_edge_dev(tri_row, 3u * j + m);
            const int ka = edge_a(e), kb = edge_b(e);
            const uint32_t ba = (uint32_t)(corner_x(ka) | (corner_y(ka) << 1) | (corner_z(ka) << 2));
            const uint32_t bb = (uint32_t)(corner_x(kb) | (corner_y(kb) << 1) | (corner_z(kb) << 2));
            v[m] = edge_point_plain_v(sel8(c, ka), sel8(c, kb), corner_sel(V, ba), corner_sel(V, bb), p.iso);
          }
          const float3 n = normal_of(v[0], v[1], v[2]);
          const uint64_t idx = 3ull * (E.first[slot] + j);
          if (idx + 3 > p.capacity) {
            dropped = true;
            continue;
          }
#pragma unroll
          for (int m = 0; m < 3; ++m) {
            __stcs(p.pos + idx + m, make_float4(v[m].x, v[m].y, v[m].z, 1.0f));
            __stcs(p.norm + idx + m, make_float4(n.x, n.y, n.z, 0.0f));
          }
        }
    }
  }
  if (dropped) set_status(p.status, kStatusOverflow);
}

cudaError_t launch_window_count(const float* f, uint32_t nx, uint32_t ny, uint32_t nz, float iso, uint32_t* win_tris,
                                gcm_counts* counts, uint32_t blocks, cudaStream_t st, TileStates tiles) {
  if (win_tris) mc_window_count_kernel<true><<<blocks, 256, 0, st>>>(f, nx, ny, nz, iso, win_tris, counts, tiles);
  else mc_window_count_kernel<false><<<blocks, 256, 0, st>>>(f, nx, ny, nz, iso, nullptr, counts, tiles);
  return cudaGetLastError();
}

cudaError_t launch_window_emit(const WindowEmitParams& p, uint32_t blocks, cudaStream_t st) {
  mc_window_emit_kernel<<<blocks, kEmitWarps * 32, 0, st>>>(p);
  return cudaGetLastError();
}

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
// Retained primitive accumulation (classify_copy_Voxel, static mode,
// src/MarchingCubes_kernel.cu:158-447): per sample the sign becomes -1 or 1
// by the boolean of the new field f and the old sign (union: f < iso or
// val < iso; difference: f >= iso and val < iso; intersection: f < iso and
// val < iso), and on each of the sample's +x, +y, +z edges that f crosses the
// crossing fraction t = (iso - f) / (f' - f) replaces a non-positive stored
// fraction or is averaged with a positive one.  Like the reference, the last
// sample of the grid is left as it is.
// classify_copy_Voxel (src/MarchingCubes_kernel.cu:158-447): static mode (the
// field is the object) or, with `band`, the lattice-band mode (dynamic = true:
// the open band iso1 < f < iso2 is the object, the crossing fraction is taken
// at iso1, else at iso2, and the difference pairs the band with the old
// outside as the reference does).
__global__ void __launch_bounds__(256) csg_retain_kernel(gcm_csg_point* __restrict__ acc, const float* __restrict__ f,
                                                         uint32_t nx, uint32_t ny, uint32_t nz, float iso, uint32_t op,
                                                         bool band, float iso1, float iso2) {
  const uint64_t plane = (uint64_t)nx * ny, total = plane * nz;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i + 1 < total;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t x = (uint32_t)(i % nx), y = (uint32_t)((i / nx) % ny), z = (uint32_t)(i / plane);
    gcm_csg_point pt = acc[i];
    const float v = __ldg(f + i);
    const bool in_a = (float)pt.val < iso;
    bool inside;
    if (band) {
      const bool in_b = (v > iso1) && (v < iso2);
      if (op == GCM_CSG_SUBTRACT) inside = in_b && !in_a;
      else if (op == GCM_CSG_INTERSECT) inside = in_b && in_a;
      else inside = in_b || in_a;
    } else {
      const bool in_v = v < iso;
      if (op == GCM_CSG_SUBTRACT) inside = (v >= iso) && in_a;
      else if (op == GCM_CSG_INTERSECT) inside = in_v && in_a;
      else inside = in_v || in_a;
    }
    pt.val = inside ? -1 : 1;
    auto crosses = [&](float w, float lev) { return (w < lev && v >= lev) || (w >= lev && v < lev); };
    auto fold = [&](float& ts, float w) {
      float lev;
      if (!band) {
        if (!crosses(w, iso)) return;
        lev = iso;
      } else if (crosses(w, iso1)) {
        lev = iso1;
      } else if (crosses(w, iso2)) {
        lev = iso2;
      } else {
        return;
      }
      const float t = __fdiv_rn(__fsub_rn(lev, v), __fsub_rn(w, v));
      ts = ts > 0.0f ? __fmul_rn(__fadd_rn(ts, t), 0.5f) : t;
    };
    if (x + 1 < nx) fold(pt.t_x, __ldg(f + i + 1));
    if (y + 1 < ny) fold(pt.t_y, __ldg(f + i + nx));
    if (z + 1 < nz) fold(pt.t_z, __ldg(f + i + plane));
    acc[i] = pt;
  }
}

using MeshFn = void (*)(MeshParams, MeshLayout);
template <int M, int T>
MeshFn mesh_fn_e(bool emit) {
  return emit ? mc_mesh_kernel<M, true, T> : mc_mesh_kernel<M, false, T>;
}
template <int T>
MeshFn mesh_fn_t(int mode, bool emit) {
  switch (mode) {
    case kMeshBand: return mesh_fn_e<kMeshBand, T>(emit);
    case kMeshRegion: return mesh_fn_e<kMeshRegion, T>(emit);
    case kMeshPreview: return mesh_fn_e<kMeshPreview, T>(emit);
    case kMeshLatFixed: return mesh_fn_e<kMeshLatFixed, T>(emit);
    case kMeshLatDynamic: return mesh_fn_e<kMeshLatDynamic, T>(emit);
    default: return mesh_fn_e<kMeshPlain, T>(emit);
  }
}
MeshFn mesh_fn(int mode, bool emit, int threads) {
  return threads == 128 ? mesh_fn_t<128>(mode, emit) : mesh_fn_t<256>(mode, emit);
}
using BatchFn = void (*)(BatchMeshParams, MeshLayout);
BatchFn batch_fn(bool emit, int threads) {
  if (threads == 128) return emit ? mc_batch_kernel<true, 128> : mc_batch_kernel<false, 128>;
  return emit ? mc_batch_kernel<true, 256> : mc_batch_kernel<false, 256>;
}
template <class F>
cudaError_t prepare(F f, size_t smem, int threads, int* blocks_per_sm) {
  // The dynamic shared memory limit is a per-kernel, process-wide attribute:
  // it is always raised to the kernel's full opt-in limit (the same value from
  // every thread), so that concurrent callers with different tile sizes never
  // lower it under one another's launch.  Occupancy follows `smem`, not it.
  int dev = 0, optin = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaFuncAttributes fa{};
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, f);
  if (e != cudaSuccess) return e;
  const int limit = optin - (int)fa.sharedSizeBytes;
  if ((int)smem > limit) return cudaErrorInvalidValue;
  if (fa.maxDynamicSharedSizeBytes != limit) {
    e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, limit);
    if (e != cudaSuccess) return e;
  }
  // all of the unified L1/shared storage as shared memory: occupancy is
  // limited by shared memory, and the kernel reads global memory only
  // through bulk copies and read-only loads
  e = cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, f, threads, smem);
}
}  // namespace

bool mesh_threads_supported(int threads) { return threads == 128 || threads == 256; }

cudaError_t mesh_prepare(int mode, bool emit, int threads, size_t smem, int* blocks_per_sm) {
  return prepare(mesh_fn(mode, emit, threads), smem, threads, blocks_per_sm);
}

cudaError_t launch_mesh(int mode, bool emit, int threads, const MeshParams& p, const MeshLayout& L, uint32_t blocks,
                        cudaStream_t st) {
  mesh_fn(mode, emit, threads)<<<blocks, threads, L.total, st>>>(p, L);
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

cudaError_t launch_csg_retain(gcm_csg_point* acc, const float* f, uint32_t nx, uint32_t ny, uint32_t nz, float iso,
                              uint32_t op, bool band, float iso1, float iso2, uint32_t blocks, cudaStream_t st) {
  csg_retain_kernel<<<blocks, 256, 0, st>>>(acc, f, nx, ny, nz, iso, op, band, iso1, iso2);
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
  if (((reinterpret_cast<uintptr_t>(p.in) | reinterpret_cast<uintptr_t>(p.out)) & 15u) == 0)
    scan_u32_kernel<true><<<blocks, kScanThreads, 0, st>>>(p);
  else
    scan_u32_kernel<false><<<blocks, kScanThreads, 0, st>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_lookback_stall(uint32_t ntiles, uint32_t stall, uint64_t wait_ns, uint64_t* tile_status,
                                  uint32_t* counter, uint64_t* prefix_out, uint32_t* status, uint32_t blocks,
                                  cudaStream_t st) {
  lookback_stall_kernel<<<blocks, 32, 0, st>>>(ntiles, stall, wait_ns, tile_status, counter, prefix_out, status);
  return cudaGetLastError();
}

}  // namespace gcm
