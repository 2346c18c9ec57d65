// Device-side building blocks shared by the meshing kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "mc_tables.h"

namespace gcm {

// Status codes written by kernels into gcm_counts::status (same values as gcm.h).
enum : uint32_t { kStatusOk = 0, kStatusOverflow = 2, kStatusTimeout = 3, kStatusInvalid = 1 };

// The triangle table in global memory; every CTA copies it to shared memory,
// where the data-dependent row lookups of a warp do not serialise.
static __device__ const uint64_t g_tri_rows[256] = {GCM_TRI_ROWS};

__device__ __forceinline__ void load_tri_table(uint64_t* s_tri) {
  for (int i = threadIdx.x; i < 256; i += blockDim.x) s_tri[i] = g_tri_rows[i];
}

// Number of vertices of a configuration = 3 x triangles: the row's leading
// non-0xF nibbles (trailing 0xF nibbles counted from the low end).
__device__ __forceinline__ uint32_t row_nverts(uint64_t row) {
  const uint64_t inv = ~row;
  if (inv == 0) return 0;
  return 16u - (uint32_t)(__ffsll((long long)inv) - 1) / 4u;
}
__device__ __forceinline__ uint32_t row_ntris(uint64_t row) { return row_nverts(row) / 3u; }

// The fused kernel's copy of the table: the lowest nibble of every row (the
// 0xF terminator in every configuration, which has at most 15 edge entries)
// holds the configuration's triangle count instead, so `row & 0xF` is the
// count and the edge nibbles of triangles 0..4 are unchanged.
__device__ __forceinline__ void load_tri_table_counted(uint64_t* s_tri) {
  for (int i = threadIdx.x; i < 256; i += blockDim.x) {
    const uint64_t r = g_tri_rows[i];
    s_tri[i] = (r & ~0xFull) | row_ntris(r);
  }
}

// Edges 3j, 3j+1, 3j+2 of triangle j (j < 5) as a 12-bit group, first edge in
// the top nibble.
__device__ __forceinline__ uint32_t tri_edges3(uint64_t row, uint32_t j) {
  return (uint32_t)(row >> (52u - 12u * j)) & 0xFFFu;
}

__device__ __forceinline__ uint32_t tri_edge_dev(uint64_t row, uint32_t j) {
  return (uint32_t)((row >> (4u * (15u - j))) & 0xFu);
}

// --------------------------------------------------------------------------
// Vertex arithmetic.  The reference forms p = (gridPos - gridcenter) *
// voxelSize, corners p + offset, edge points lerp(va, vb, t) with
// t = (iso - fa) / (fb - fa), and normals cross(v1 - v0, v2 - v0)
// (src/MarchingCubes_kernel.cu:3061-3075, 1619-1637; helper_math.h:1145-1148,
// 1427-1430).  nvcc contracts that source into the rounding pattern below
// (corner and delta unfused, lerp fma(t, b - a, a), cross terms
// fma(a, b, -(c*d))); it is identified from the reference's compiled kernels
// and written out with explicit IEEE intrinsics so no later compiler change can
// alter it.
// --------------------------------------------------------------------------

struct Frame {
  float vs[3];
  float gc[3];
};

__device__ __forceinline__ float corner_coord(uint32_t g, float gc, float vs, int off) {
  const float P = __fmul_rn(__fsub_rn(__uint2float_rn(g), gc), vs);
  return off ? __fadd_rn(P, vs) : P;
}

__device__ __forceinline__ float lerp_coord(float a, float b, float t) {
  return __fmaf_rn(t, __fsub_rn(b, a), a);
}

__device__ __forceinline__ float cross_term(float a, float b, float c, float d) {
  return __fmaf_rn(a, b, -__fmul_rn(c, d));
}

__device__ __forceinline__ float3 normal_of(float3 v0, float3 v1, float3 v2) {
  const float3 e0 = make_float3(__fsub_rn(v1.x, v0.x), __fsub_rn(v1.y, v0.y), __fsub_rn(v1.z, v0.z));
  const float3 e1 = make_float3(__fsub_rn(v2.x, v0.x), __fsub_rn(v2.y, v0.y), __fsub_rn(v2.z, v0.z));
  return make_float3(cross_term(e0.y, e1.z, e0.z, e1.y), cross_term(e0.z, e1.x, e0.x, e1.z),
                     cross_term(e0.x, e1.y, e0.y, e1.x));
}

__device__ __forceinline__ float3 corner_pos(const uint32_t g[3], const Frame& fr, int k) {
  return make_float3(corner_coord(g[0], fr.gc[0], fr.vs[0], corner_x(k)),
                     corner_coord(g[1], fr.gc[1], fr.vs[1], corner_y(k)),
                     corner_coord(g[2], fr.gc[2], fr.vs[2], corner_z(k)));
}

__device__ __forceinline__ float3 lerp3(float3 a, float3 b, float t) {
  return make_float3(lerp_coord(a.x, b.x, t), lerp_coord(a.y, b.y, t), lerp_coord(a.z, b.z, t));
}

// The two candidate coordinates of a voxel's corners on each axis:
// corner_coord(g, gc, vs, 0) and corner_coord(g, gc, vs, 1).
struct VoxelCorners {
  float x0, x1, y0, y1, z0, z1;
};

__device__ __forceinline__ void axis_corners(uint32_t g, float gc, float vs, float& c0, float& c1) {
  c0 = corner_coord(g, gc, vs, 0);
  c1 = corner_coord(g, gc, vs, 1);
}

// Corner with bits (x | y << 1 | z << 2): equal to corner_pos for that corner.
__device__ __forceinline__ float3 corner_sel(const VoxelCorners& V, uint32_t bits) {
  return make_float3((bits & 1u) ? V.x1 : V.x0, (bits & 2u) ? V.y1 : V.y0, (bits & 4u) ? V.z1 : V.z0);
}

// Plain edge point from the two corner values and positions (the same
// arithmetic as edge_point_plain).
__device__ __forceinline__ float3 edge_point_plain_v(float fa, float fb, float3 pa, float3 pb, float iso) {
  const float t = __fdiv_rn(__fsub_rn(iso, fa), __fsub_rn(fb, fa));
  return lerp3(pa, pb, t);
}

// Plain edge point (vertexInterp4, src/MarchingCubes_kernel.cu:1619-1629).
// `val(k)` returns the field at corner k; only the edge's two corners are read,
// so no per-voxel corner array is indexed at run time.
template <class Val>
__device__ __forceinline__ float3 edge_point_plain(const uint32_t g[3], const Frame& fr, uint32_t e, Val&& val,
                                                   float iso) {
  const int ka = edge_a((int)e), kb = edge_b((int)e);
  const float fa = val(ka), fb = val(kb);
  const float t = __fdiv_rn(__fsub_rn(iso, fa), __fsub_rn(fb, fa));
  return lerp3(corner_pos(g, fr, ka), corner_pos(g, fr, kb), t);
}

// The reference compares float differences against the double 0.0005
// ((double)|d| < 0.0005).  float(0.0005) = 5.000000237e-4 is the smallest float
// above 0.0005, so for every float d, |d| < float(0.0005) gives the same
// answer (NaN included) without the FP64 pipe.
constexpr float kSnap = 0.0005f;

// Band edge point (vertexInterp2_new, src/MarchingCubes_kernel.cu:3593-3674):
// endpoints with labels {0,1} are ordered so that f0 <= f1; the point snaps to
// an endpoint within 0.0005 of a band edge (the reference's double comparison,
// made exactly in float through kSnap) and otherwise lerps at the band edge
// crossed.  Where the reference leaves t unset, t = 0.  `lab(k)` / `fv(k)`
// return the label and the normalised field at corner k.
template <class Lab, class Fv>
__device__ __forceinline__ float3 edge_point_band(const uint32_t g[3], const Frame& fr, uint32_t e, Lab&& lab, Fv&& fv,
                                                  float lo, float hi) {
  int ka = edge_a((int)e), kb = edge_b((int)e);
  const float id0 = lab(ka), id1 = lab(kb);
  float f0 = fv(ka), f1 = fv(kb);
  const bool crossing = (id0 == 1.0f && id1 == 0.0f) || (id0 == 0.0f && id1 == 1.0f);
  if (crossing && f1 < f0) {
    const int tk = ka; ka = kb; kb = tk;
    const float tf = f0; f0 = f1; f1 = tf;
  }
  const float3 pa = corner_pos(g, fr, ka), pb = corner_pos(g, fr, kb);
  float t = 0.0f;
  if (crossing) {
    bool done = false;
#pragma unroll
    for (int side = 0; side < 2; ++side) {
      const float lev = side ? hi : lo;
      if (!done && (f1 >= lev) && (f0 <= lev)) {
        if (fabsf(__fsub_rn(lev, f0)) < kSnap) return pa;
        if (fabsf(__fsub_rn(lev, f1)) < kSnap) return pb;
        if (fabsf(__fsub_rn(f1, f0)) < kSnap) return pa;
        t = __fdiv_rn(__fsub_rn(lev, f0), __fsub_rn(f1, f0));
        done = true;
      }
    }
    if (!done) {
      if ((f1 == f0) && (pa.z == 0.0f)) t = 1.0f;
      else if (f1 == f0) t = 0.0f;
    }
  }
  return lerp3(pa, pb, t);
}

// Band edge point from the corner labels, normalised values and corner bits
// (the same arithmetic and branch order as edge_point_band).
__device__ __forceinline__ float3 edge_point_band_v(float id0, float id1, float f0, float f1, uint32_t ba, uint32_t bb,
                                                    const VoxelCorners& V, float lo, float hi) {
  // The reference's branches as selects: the first band edge crossed (lo,
  // then hi) decides the level; snapping returns an end point exactly; the
  // interpolation is made with the same operations either way.
  const bool crossing = (id0 == 1.0f && id1 == 0.0f) || (id0 == 0.0f && id1 == 1.0f);
  const bool swap = crossing && f1 < f0;
  const uint32_t ua = swap ? bb : ba, ub = swap ? ba : bb;
  const float g0 = swap ? f1 : f0, g1 = swap ? f0 : f1;
  const float3 pa = corner_sel(V, ua), pb = corner_sel(V, ub);
  const bool on_lo = (g1 >= lo) && (g0 <= lo), on_hi = (g1 >= hi) && (g0 <= hi);
  const bool hit = crossing && (on_lo || on_hi);
  const float lev = on_lo ? lo : hi;
  const float d0 = __fsub_rn(lev, g0), d1 = __fsub_rn(lev, g1), dd = __fsub_rn(g1, g0);
  const bool s0 = fabsf(d0) < kSnap, s1 = fabsf(d1) < kSnap, s2 = fabsf(dd) < kSnap;
  float t = 0.0f;
  if (hit) t = __fdiv_rn(d0, dd);
  else if (crossing && g1 == g0) t = pa.z == 0.0f ? 1.0f : 0.0f;
  const float3 p = lerp3(pa, pb, t);
  if (hit && (s0 || (!s1 && s2))) return pa;
  if (hit && !s0 && s1) return pb;
  return p;
}

// Lattice "fixed" preview edge point (vertexInterp_new, src/MarchingCubes_kernel.cu:
// 1728-1790): fractions where the primitive field f crosses iso and where the
// lattice L crosses lo and hi (strict on the lower side), combined as the
// reference does; (t1 + t) * 0.5 runs in double there, which rounds to the
// same float as the float product.
__device__ __forceinline__ float3 edge_point_latfixed(float iso, float lo, float hi, float3 pa, float3 pb, float f0,
                                                      float f1, float l0, float l1) {
  float t1 = 0.0f, t2 = 0.0f, t3 = 0.0f;
  if (((f0 < iso) && (f1 >= iso)) || ((f1 < iso) && (f0 >= iso))) t1 = __fdiv_rn(__fsub_rn(iso, f0), __fsub_rn(f1, f0));
  if (((l0 < lo) && (l1 >= lo)) || ((l1 < lo) && (l0 >= lo))) t2 = __fdiv_rn(__fsub_rn(lo, l0), __fsub_rn(l1, l0));
  if (((l0 < hi) && (l1 >= hi)) || ((l1 < hi) && (l0 >= hi))) t3 = __fdiv_rn(__fsub_rn(hi, l0), __fsub_rn(l1, l0));
  float t = 0.0f;
  if ((t1 > 0.0f) && (t2 > 0.0f) && (t3 == 0.0f)) t = __fmul_rn(__fadd_rn(t1, t2), 0.5f);
  else if ((t1 > 0.0f) && (t3 > 0.0f) && (t2 == 0.0f)) t = __fmul_rn(__fadd_rn(t1, t3), 0.5f);
  else if ((t1 > 0.0f) && (t2 == 0.0f) && (t3 == 0.0f)) t = t1;
  else if ((t2 > 0.0f) && (t1 == 0.0f) && (t3 == 0.0f)) t = t2;
  else if ((t3 > 0.0f) && (t1 == 0.0f) && (t2 == 0.0f)) t = t3;
  return lerp3(pa, pb, t);
}

// Lattice "dynamic" preview edge point (vertexInterp_primitive_one,
// src/MarchingCubes_kernel.cu:1676-1726): the stored fraction t1 of the edge's
// lower corner combined with where the lattice crosses lo, then (overriding
// where it applies) with where it crosses hi; inclusive crossing tests.
__device__ __forceinline__ float3 edge_point_latdyn(float lo, float hi, float3 p0, float3 p1, float l0, float l1,
                                                    float t1) {
  float t2 = 0.0f, t3 = 0.0f, t = 0.0f;
  if (((l1 >= lo) && (l0 <= lo)) || ((l0 >= lo) && (l1 <= lo))) t2 = __fdiv_rn(__fsub_rn(lo, l0), __fsub_rn(l1, l0));
  if ((t1 > 0.0f) && (t2 > 0.0f)) t = __fmul_rn(__fadd_rn(t1, t2), 0.5f);
  else if ((t1 > 0.0f) && (t2 == 0.0f)) t = t1;
  else if ((t2 > 0.0f) && (t1 == 0.0f)) t = t2;
  if (((l1 >= hi) && (l0 <= hi)) || ((l0 >= hi) && (l1 <= hi))) t3 = __fdiv_rn(__fsub_rn(hi, l0), __fsub_rn(l1, l0));
  if ((t1 > 0.0f) && (t3 > 0.0f)) t = __fmul_rn(__fadd_rn(t1, t3), 0.5f);
  else if ((t1 > 0.0f) && (t3 == 0.0f)) t = t1;
  else if ((t3 > 0.0f) && (t1 == 0.0f)) t = t3;
  return lerp3(p0, p1, t);
}

// Retained edge point (vertexInterp_primitive, src/MarchingCubes_kernel.cu:
// 1640-1672): the crossing fraction t2 of the fed field on the edge (inclusive
// tests on both sides), averaged with the accumulated fraction t1 when both
// are positive, else whichever is positive alone, else 0; p0 is the edge's
// lower corner.  (t1 + t2) * 0.5 runs in double in the reference, which rounds
// to the same float as the float product.
__device__ __forceinline__ float3 edge_point_retained(float iso, float3 p0, float3 p1, float f0, float f1, float t1) {
  float t2 = 0.0f;
  if (((f1 >= iso) && (f0 <= iso)) || ((f0 >= iso) && (f1 <= iso))) t2 = __fdiv_rn(__fsub_rn(iso, f0), __fsub_rn(f1, f0));
  float t = 0.0f;
  if ((t1 > 0.0f) && (t2 > 0.0f)) t = __fmul_rn(__fadd_rn(t1, t2), 0.5f);
  else if ((t1 > 0.0f) && (t2 == 0.0f)) t = t1;
  else if ((t2 > 0.0f) && (t1 == 0.0f)) t = t2;
  return lerp3(p0, p1, t);
}

__device__ __forceinline__ uint32_t cube_index8(const float c[8], float iso) {
  uint32_t ci = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) ci |= (uint32_t)(c[k] < iso) << k;
  return ci;
}

// --------------------------------------------------------------------------
// Warp helpers.
// --------------------------------------------------------------------------
__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
  const uint32_t lane = threadIdx.x & 31u;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t n = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= (uint32_t)o) v += n;
  }
  return v;
}

__device__ __forceinline__ uint64_t warp_sum_u64(uint64_t v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Lanes below this one, as a mask.
__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Bit planes of per-lane counts below 8 (three ballots): a lane's exclusive
// prefix is sum_k 2^k popc(plane_k & lanes below), the warp's total
// sum_k 2^k popc(plane_k).
struct CountPlanes {
  uint32_t b0, b1, b2;
};
__device__ __forceinline__ CountPlanes count_planes(uint32_t v) {
  return {__ballot_sync(0xffffffffu, v & 1u), __ballot_sync(0xffffffffu, v & 2u), __ballot_sync(0xffffffffu, v & 4u)};
}
__device__ __forceinline__ uint32_t planes_total(const CountPlanes& c) {
  return (uint32_t)__popc(c.b0) + 2u * (uint32_t)__popc(c.b1) + 4u * (uint32_t)__popc(c.b2);
}
__device__ __forceinline__ uint32_t planes_excl(const CountPlanes& c) {
  const uint32_t lt = lanemask_lt();
  return (uint32_t)__popc(c.b0 & lt) + 2u * (uint32_t)__popc(c.b1 & lt) + 4u * (uint32_t)__popc(c.b2 & lt);
}

__device__ __forceinline__ uint64_t global_timer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void set_status(uint32_t* status, uint32_t code) {
  if (status) atomicCAS(status, 0u, code);
}

// --------------------------------------------------------------------------
// Decoupled look-back over tiles processed in increasing order.  Each tile's
// status word holds (flag << 62) | value: flag 1 = the tile's own aggregate,
// flag 2 = inclusive prefix through that tile.  Waiting is bounded by wall
// time; on expiry the status is set to timeout and 0 is used as the prefix.
// Called by one full warp; returns the exclusive prefix on every lane.
// --------------------------------------------------------------------------
constexpr uint64_t kFlagAgg = 1ull << 62;
constexpr uint64_t kFlagPre = 2ull << 62;
constexpr uint64_t kValMask = (1ull << 62) - 1;

__device__ __forceinline__ uint64_t ld_status(const uint64_t* p) {
  uint64_t v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_status(uint64_t* p, uint64_t v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ uint64_t lookback_exclusive(uint64_t* status, uint64_t tile, uint64_t aggregate,
                                                       uint64_t wait_ns, uint32_t* err) {
  const uint32_t lane = threadIdx.x & 31u;
  if (tile == 0) {
    if (lane == 0) st_status(&status[0], kFlagPre | aggregate);
    return 0;
  }
  if (lane == 0) st_status(&status[tile], kFlagAgg | aggregate);
  uint64_t excl = 0;
  int64_t base = (int64_t)tile - 1;
  const uint64_t t0 = global_timer_ns();
  uint32_t spins = 0;
  while (true) {
    const int64_t i = base - (int64_t)lane;
    const uint64_t w = (i >= 0) ? ld_status(&status[i]) : kFlagPre;
    const uint32_t flag = (uint32_t)(w >> 62);
    const uint32_t pmask = __ballot_sync(0xffffffffu, flag == 2u);
    const uint32_t imask = __ballot_sync(0xffffffffu, flag == 0u);
    const int first_p = pmask ? __ffs((int)pmask) - 1 : 32;
    const uint32_t before = first_p == 32 ? 0xffffffffu : ((1u << first_p) - 1u);
    if (imask & before) {
      if (((++spins) & 63u) == 0u && global_timer_ns() - t0 > wait_ns) {
        if (lane == 0) set_status(err, kStatusTimeout);
        excl = 0;
        break;
      }
      __nanosleep(64);
      continue;
    }
    const uint64_t v = ((int)lane <= first_p) ? (w & kValMask) : 0ull;
    excl += warp_sum_u64(v);
    if (first_p < 32) break;
    base -= 32;
  }
  if (lane == 0) st_status(&status[tile], kFlagPre | ((excl + aggregate) & kValMask));
  return excl;
}

// --------------------------------------------------------------------------
// Bulk (TMA) copies global -> shared with an mbarrier.
// --------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for one phase of the barrier; false if it ran out of time.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint64_t wait_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_timer_ns();
  while (!mbar_try_wait(bar, parity)) {
    if (global_timer_ns() - t0 > wait_ns) return false;
  }
  return true;
}

}  // namespace gcm
