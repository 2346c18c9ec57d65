// Spatially variant lattices (SVL) for sm_103a: the reference's Fourier-grating
// lattice synthesis (src/main.cu:3578-3711, 3904-4030; src/lattice_files/
// Gratings.cu:100-1050).
//
// A unit-cell TPMS is expanded in Fourier coefficients c_ijk; for each of the
// first n_coeff coefficients a phase field phi_ijk is solved on the control
// grid from the locally rotated and scaled grating vector (finding_phi_kernel
// gives the right-hand side, GPUCG_lattice the conjugate-gradient solve), and
// the lattice on the twice-finer grid is the sum of Re(c_ijk exp(i phi_ijk)).
//
// GB300 form: every coefficient's system has the same matrix, so all n_coeff
// solves run together, one kernel per CG step for all of them, with the
// scalars of each solve kept on the device (no host round trip per step) and
// the steps replayed from a CUDA graph.  Dot products use the reference's
// partition and order (1024-element blocks reduced as a tree, then one
// 1024-thread block adding its strided partials in sequence and reducing as a
// tree), and every other operation is written in the reference's rounding
// pattern, so each solve's iterates are its iterates.  The coefficients come
// from a direct DFT of the unit cell at the (2 range + 1)^3 frequencies used.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <vector>

#include "../../include/gcm.h"
#include "gcm_ctx.h"
#include "gcm_kernels.h"

namespace gcm {
namespace {

constexpr int kBlock = 1024;  // the reference's reduction block

struct SvlGeo {
  int nx, ny, nz;
  float dx, dy, dz;
  uint32_t kind, period_type;
  float period, px, py, pz, lcon, lcon_1;
  uint32_t sinewave_z;
};

struct Freq {
  int i, j, k;
};

// Frequencies of coefficient m in the reference's order: k outer, j, i inner,
// each over [-range, range] (src/main.cu:3615-3690).
__host__ __device__ inline Freq freq_of(uint32_t m, int range) {
  const int w = 2 * range + 1;
  Freq f;
  f.i = (int)(m % w) - range;
  f.j = (int)((m / w) % w) - range;
  f.k = (int)(m / (w * w)) - range;
  return f;
}

// One-sided / central difference weights of the reference along one axis
// (finding_phi_kernel, Gratings.cu:139-241): (a1, a2) and neighbours (x1, x2).
struct Stencil1 {
  float a1, a2;
  int n1, n2;
};
__device__ __forceinline__ Stencil1 stencil1(int x, int n) {
  Stencil1 s;
  if (x == 0) { s.a1 = -1.0f; s.a2 = -0.5f; s.n1 = x; s.n2 = x + 1; }
  else if (x == 1) { s.a1 = 1.0f; s.a2 = -0.5f; s.n1 = x - 1; s.n2 = x + 1; }
  else if (x == n - 2) { s.a1 = 0.5f; s.a2 = -1.0f; s.n1 = x - 1; s.n2 = x + 1; }
  else if (x == n - 1) { s.a1 = 0.5f; s.a2 = 1.0f; s.n1 = x - 1; s.n2 = x; }
  else { s.a1 = 0.5f; s.a2 = -0.5f; s.n1 = x - 1; s.n2 = x + 1; }
  return s;
}

// (2 pi / per) * v in double, rounded to float, as the reference's
// ((2*M_PI)/per)*(float expression) is.
__device__ __forceinline__ float kscale(float per, float v) {
  return (float)((2.0 * 3.14159265358979323846 / (double)per) * (double)v);
}

// i * c - j * s and i * s + j * c as nvcc contracts them in the reference.
__device__ __forceinline__ float rot_a(int i, int j, float c, float s) {
  return __fmaf_rn((float)i, c, -__fmul_rn((float)j, s));
}
__device__ __forceinline__ float rot_b(int i, int j, float c, float s) {
  return __fmaf_rn((float)i, s, __fmul_rn((float)j, c));
}

// Right-hand sides of every coefficient at every control sample
// (finding_phi_kernel, Gratings.cu:100-417).  The sample's geometry (stencil
// weights, rotation angles, periods) is made once and reused for each
// coefficient.  Also initialises each solve: d = r = rhs, x = 0.
__global__ void __launch_bounds__(256) svl_rhs_kernel(SvlGeo g, const float* __restrict__ d_period, int range,
                                                      uint32_t n_coeff, uint64_t P, float* __restrict__ x,
                                                      float* __restrict__ r, float* __restrict__ d) {
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < P; t += (uint64_t)gridDim.x * blockDim.x) {
    const int tx = (int)t;
    const int X = g.nx, Y = g.ny, Z = g.nz;
    const int xi = tx % X, yi = (tx % (X * Y)) / X, zi = tx / (X * Y);
    const Stencil1 sx = stencil1(xi, X), sy = stencil1(yi, Y), sz = stencil1(zi, Z);
    float th1 = 0.0f, th2 = 0.0f, th3 = 0.0f, th4 = 0.0f, th5 = 0.0f, th6 = 0.0f, th7 = 0.0f, th8 = 0.0f;
    const float con = 1.0f, angl = 0.0f;
    if (g.kind == 'r' || g.kind == 'b') {
      const float mx = g.kind == 'r' ? (float)(X + 1) / 2.0f : 0.0f;
      const float my = g.kind == 'r' ? (float)(Y + 1) / 2.0f : 0.0f;
      const float yy = __fmul_rn(__fsub_rn((float)(yi + 1), my), g.dx);
      const float xx1 = __fmul_rn(__fsub_rn((float)(sx.n1 + 1), mx), g.dx);
      const float xx2 = __fmul_rn(__fsub_rn((float)(sx.n2 + 1), mx), g.dx);
      th1 = atan2f(yy, xx1);
      th2 = atan2f(yy, xx2);
      const float xx = __fmul_rn(__fsub_rn((float)(xi + 1), mx), g.dx);
      const float yy1 = __fmul_rn(__fsub_rn((float)(sy.n1 + 1), my), g.dx);
      const float yy2 = __fmul_rn(__fsub_rn((float)(sy.n2 + 1), my), g.dx);
      th3 = atan2f(yy1, xx);
      th4 = atan2f(yy2, xx);
    } else if (g.kind == 's') {
      // lcon * sinf(6.28 * lcon_1 * u): the argument in double
      auto wave = [&](float u) { return __fmul_rn(g.lcon, sinf((float)(6.28 * (double)g.lcon_1 * (double)u))); };
      const float xx1 = __fmul_rn((float)(sx.n1 + 1), g.dx), zz1 = __fmul_rn((float)(sz.n1 + 1), g.dz);
      const float xx2 = __fmul_rn((float)(sx.n2 + 1), g.dx), zz2 = __fmul_rn((float)(sz.n2 + 1), g.dz);
      const float xx = __fmul_rn((float)(xi + 1), g.dx), zz = __fmul_rn((float)(zi + 1), g.dz);
      th1 = wave(xx1);
      th5 = wave(zz1);
      th2 = wave(xx2);
      th6 = wave(zz2);
      th3 = wave(xx);
      th7 = wave(zz);
      th4 = th3;
      th8 = th7;
    }
    float p1, p2, p3, p4, p5, p6;
    if (g.period_type == 1) {
      p1 = p2 = g.px;
      p3 = p4 = g.py;
      p5 = p6 = g.pz;
    } else if (g.period_type == 2) {
      const int XY = X * Y;
      p1 = __ldg(d_period + sx.n1 + yi * X + zi * XY);
      p2 = __ldg(d_period + sx.n2 + yi * X + zi * XY);
      p3 = __ldg(d_period + xi + sy.n1 * X + zi * XY);
      p4 = __ldg(d_period + xi + sy.n2 * X + zi * XY);
      p5 = __ldg(d_period + xi + yi * X + sz.n1 * XY);
      p6 = __ldg(d_period + xi + yi * X + sz.n2 * XY);
    } else {
      p1 = p2 = p3 = p4 = p5 = p6 = g.period;
    }
    const float c1 = cosf(th1), s1 = sinf(th1), c2 = cosf(th2), s2 = sinf(th2);
    const float c3 = cosf(th3), s3 = sinf(th3), c4 = cosf(th4), s4 = sinf(th4);
    for (uint32_t m = 0; m < n_coeff; ++m) {
      const Freq q = freq_of(m, range);
      const float kx1 = kscale(p1, rot_a(q.i, q.j, c1, s1)), kx2 = kscale(p2, rot_a(q.i, q.j, c2, s2));
      const float ky1 = kscale(p3, rot_b(q.i, q.j, c3, s3)), ky2 = kscale(p4, rot_b(q.i, q.j, c4, s4));
      const float kz1 = (float)((2.0 * 3.14159265358979323846 / (double)p5) * (double)q.k);
      const float kz2 = (float)((2.0 * 3.14159265358979323846 / (double)p6) * (double)q.k);
      // the products with the stencil weights (0.5, 1, powers of two) are
      // exact, so each pair is one rounded sum
      float phii = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(sx.a1, kx1), __fmul_rn(sx.a2, kx2)),
                                       __fadd_rn(__fmul_rn(sy.a1, ky1), __fmul_rn(sy.a2, ky2))),
                             __fadd_rn(__fmul_rn(sz.a1, kz1), __fmul_rn(sz.a2, kz2)));
      if (g.kind == 's' && g.sinewave_z) {
        const float s5 = sinf(th5), s6 = sinf(th6), c7 = cosf(th7), c8 = cosf(th8);
        const float kz1b = kscale(p5, __fmaf_rn((float)q.j, s5, __fmul_rn((float)q.k, cosf(__fsub_rn(__fmul_rn(con, th5), angl)))));
        const float kz2b = kscale(p6, __fmaf_rn((float)q.j, s6, __fmul_rn((float)q.k, cosf(__fsub_rn(__fmul_rn(con, th6), angl)))));
        const float ky1b = kscale(p3, __fmaf_rn((float)q.j, c7, -__fmul_rn((float)q.k, sinf(__fadd_rn(__fmul_rn(con, th7), angl)))));
        const float ky2b = kscale(p4, __fmaf_rn((float)q.j, c8, -__fmul_rn((float)q.k, sinf(__fadd_rn(__fmul_rn(con, th8), angl)))));
        const float kx1b = (float)((2.0 * 3.14159265358979323846 / (double)p1) * (double)q.i);
        const float kx2b = (float)((2.0 * 3.14159265358979323846 / (double)p2) * (double)q.i);
        phii = __fadd_rn(phii, __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(sx.a1, kx1b), __fmul_rn(sx.a2, kx2b)),
                                                   __fadd_rn(__fmul_rn(sy.a1, ky1b), __fmul_rn(sy.a2, ky2b))),
                                         __fadd_rn(__fmul_rn(sz.a1, kz1b), __fmul_rn(sz.a2, kz2b))));
      }
      const uint64_t o = (uint64_t)m * P + t;
      r[o] = phii;
      d[o] = phii;
      x[o] = 0.0f;
    }
  }
}

// floor(n / d) for n < 2^32 as the high half of n * m, m = ceil(2^64 / d):
// the error term n * (m - 2^64 / d) / 2^64 stays below 2^-32 <= 1/d.
struct FastDiv {
  uint64_t m;
  uint32_t d;
};
inline FastDiv make_fastdiv(uint32_t d) {
  FastDiv f;
  f.d = d;
  f.m = d > 1 ? ~0ull / d + 1ull : 0ull;
  return f;
}
__device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv& f) {
  return f.d > 1 ? (uint32_t)__umul64hi((uint64_t)n, f.m) : n;
}

// A d at one control sample (GPUMatvec_lattice_kernel, Gratings.cu:420-597):
// per axis the centre weight and the two neighbour terms of the reference's
// boundary-dependent stencil; A_X = (wx + wy + wz) * d0 + the six neighbour
// terms, left to right, the first addition fused with the product.
// The five cases (c = 0, 1, n-2, n-1, interior; n >= 4) as selects of the
// neighbour offsets and weights, so boundary lanes do not diverge: each term
// is a neighbour times -1 or -0.25 (exact), as in the case-by-case form.
__device__ __forceinline__ void axis_terms(const float* dv, int c, int n, int stride, float& w, float& t2, float& t3) {
  const bool lo = c <= 1, hi = !lo && c >= n - 2;
  const int o2 = c == 0 ? stride : (c == 1 ? -stride : -2 * stride);
  const int o3 = lo ? 2 * stride : (c == n - 2 ? stride : (c == n - 1 ? -stride : 2 * stride));
  w = (lo || hi) ? 1.25f : 0.5f;
  t2 = (lo ? -1.0f : -0.25f) * dv[o2];
  t3 = (hi ? -1.0f : -0.25f) * dv[o3];
}

__device__ __forceinline__ float matvec_at(const float* __restrict__ d, int tx, int X, int Y, int Z, const FastDiv& dx,
                                           const FastDiv& dxy) {
  const int row = (int)fdiv((uint32_t)tx, dx), zi = (int)fdiv((uint32_t)tx, dxy);
  const int xi = tx - row * X, yi = row - zi * Y;
  const float* dv = d + tx;
  float wx, x2, x3, wy, y2, y3, wz, z2, z3;
  axis_terms(dv, xi, X, 1, wx, x2, x3);
  axis_terms(dv, yi, Y, X, wy, y2, y3);
  axis_terms(dv, zi, Z, X * Y, wz, z2, z3);
  float a = __fmaf_rn(__fadd_rn(__fadd_rn(wx, wy), wz), dv[0], x2);
  a = __fadd_rn(a, x3);
  a = __fadd_rn(a, y2);
  a = __fadd_rn(a, y3);
  a = __fadd_rn(a, z2);
  return __fadd_rn(a, z3);
}

// Tree reduction of one value per thread over a 1024-thread block
// (GPUScalar_lattice_kernel, Gratings.cu:600-651): levels s = 512 .. 1 add
// element t + s into element t.  The first five levels pair elements 32 w + l
// across the warp index w (pairs (w, w + 16), (w, w + 8), ... for each lane
// position l) and the last five pair the lane positions; here each is one
// warp-shuffle tree, after a transpose through padded shared memory (element
// 32 w + l at 33 w + l), so the same pairs are added in the same order with
// two barriers instead of ten.  Thread 0 returns the sum.
constexpr int kTreeSmem = kBlock + kBlock / 32 + 32;  // floats of shared memory a block_tree takes

__device__ __forceinline__ float block_tree(float v, float* cc) {
  const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
  float* rr = cc + kBlock + kBlock / 32;
  cc[threadIdx.x + w] = v;
  __syncthreads();
  float a = cc[w + 33u * lane];  // warp w now holds lane position w of every warp
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) a = __fadd_rn(a, __shfl_down_sync(0xffffffffu, a, o));
  if (lane == 0) rr[w] = a;
  __syncthreads();
  float sum = 0.0f;
  if (w == 0) {
    sum = rr[lane];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum = __fadd_rn(sum, __shfl_down_sync(0xffffffffu, sum, o));
  }
  return sum;
}

struct CgState {
  float delta_new, delta_old, alpha, beta, term;
  uint32_t active, iters;
};

// q = A d and the block partials of d . q for every active solve
// (grid: blocks x solves).
__global__ void __launch_bounds__(kBlock) svl_matvec_kernel(const float* __restrict__ d, float* __restrict__ q,
                                                            float* __restrict__ part, const CgState* st, int X, int Y,
                                                            int Z, FastDiv dx, FastDiv dxy, uint64_t P, uint32_t nblk) {
  __shared__ float cc[kTreeSmem];
  const uint32_t b = blockIdx.y;
  if (!st[b].active) return;
  const uint64_t base = (uint64_t)b * P;
  const uint64_t t = (uint64_t)blockIdx.x * kBlock + threadIdx.x;
  float c = 0.0f;
  if (t < P) {
    const float a = matvec_at(d + base, (int)t, X, Y, Z, dx, dxy);
    q[base + t] = a;
    c = __fmul_rn(d[base + t], a);
  }
  const float s = block_tree(c, cc);
  if (threadIdx.x == 0) part[(uint64_t)b * nblk + blockIdx.x] = s;
}

// Neighbour offsets and weights along one axis for sample position c (the
// selects of axis_terms), for the four-sample form.
struct AxisCase {
  int o2, o3;
  float w, k2, k3;
};
__device__ __forceinline__ AxisCase axis_case(int c, int n) {
  const bool lo = c <= 1, hi = !lo && c >= n - 2;
  AxisCase a;
  a.o2 = c == 0 ? 1 : (c == 1 ? -1 : -2);
  a.o3 = lo ? 2 : (c == n - 2 ? 1 : (c == n - 1 ? -1 : 2));
  a.w = (lo || hi) ? 1.25f : 0.5f;
  a.k2 = lo ? -1.0f : -0.25f;
  a.k3 = hi ? -1.0f : -0.25f;
  return a;
}

__device__ __forceinline__ float f4c(const float4& v, int j) { return j == 0 ? v.x : (j == 1 ? v.y : (j == 2 ? v.z : v.w)); }

// Block tree of four values per thread over a 256-thread block with the
// reference's pairs for its 1024 elements (see svl_update4_kernel); thread 0
// returns the sum.
__device__ __forceinline__ float block_tree4(float4 c, float4* cc) {
  cc[threadIdx.x] = c;
  __syncthreads();
  if (threadIdx.x >= 32) return 0.0f;
  const uint32_t lane = threadIdx.x;
  auto add4 = [](float4 u, float4 v) {
    return make_float4(__fadd_rn(u.x, v.x), __fadd_rn(u.y, v.y), __fadd_rn(u.z, v.z), __fadd_rn(u.w, v.w));
  };
  float4 v[8];
#pragma unroll
  for (int w = 0; w < 8; ++w) v[w] = cc[32 * w + lane];
#pragma unroll
  for (int h = 4; h > 0; h >>= 1)
#pragma unroll
    for (int w = 0; w < h; ++w) v[w] = add4(v[w], v[w + h]);
  float4 a = v[0];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float4 o4 = make_float4(__shfl_down_sync(0xffffffffu, a.x, o), __shfl_down_sync(0xffffffffu, a.y, o),
                                  __shfl_down_sync(0xffffffffu, a.z, o), __shfl_down_sync(0xffffffffu, a.w, o));
    a = add4(a, o4);
  }
  return __fadd_rn(__fadd_rn(a.x, a.z), __fadd_rn(a.y, a.w));
}

// q = A d and the block partials of d . q, four consecutive samples of one
// row per thread (X a multiple of 4): the x neighbours come from the 12
// values d[t-4 .. t+7] (three 16-byte loads; the outer two are needed, and
// read, only away from the row ends), the y and z neighbours from two 16-byte
// loads per axis.  Same terms, same order as matvec_at.
__global__ void __launch_bounds__(kBlock / 4) svl_matvec4_kernel(const float* __restrict__ d, float* __restrict__ q,
                                                                 float* __restrict__ part, const CgState* st, int X,
                                                                 int Y, int Z, FastDiv dx, FastDiv dxy, uint64_t P,
                                                                 uint32_t nblk) {
  __shared__ float4 cc[kBlock / 4];
  const uint32_t b = blockIdx.y;
  if (!st[b].active) return;
  const uint64_t base = (uint64_t)b * P;
  const uint64_t t = 4ull * ((uint64_t)blockIdx.x * (kBlock / 4) + threadIdx.x);
  float4 c = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  if (t < P) {
    const float* dv = d + base + t;
    const int row = (int)fdiv((uint32_t)t, dx), zi = (int)fdiv((uint32_t)t, dxy);
    const int x0 = (int)t - row * X, yi = row - zi * Y, XY = X * Y;
    const float4 mid = *reinterpret_cast<const float4*>(dv);
    const float4 left = x0 > 0 ? *reinterpret_cast<const float4*>(dv - 4) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const float4 right = x0 + 4 < X ? *reinterpret_cast<const float4*>(dv + 4) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    auto win = [&](int k) {  // d[t + k - 4], k in [0, 12)
      return k < 4 ? f4c(left, k) : (k < 8 ? f4c(mid, k - 4) : f4c(right, k - 8));
    };
    const AxisCase ay = axis_case(yi, Y), az = axis_case(zi, Z);
    const float4 y2v = *reinterpret_cast<const float4*>(dv + ay.o2 * X);
    const float4 y3v = *reinterpret_cast<const float4*>(dv + ay.o3 * X);
    const float4 z2v = *reinterpret_cast<const float4*>(dv + (int64_t)az.o2 * XY);
    const float4 z3v = *reinterpret_cast<const float4*>(dv + (int64_t)az.o3 * XY);
    float a[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const AxisCase ax = axis_case(x0 + j, X);
      // the x neighbours at offsets o2, o3 in {-2, -1, +1, +2}, as selects
      const float n2 = ax.o2 == 1 ? win(5 + j) : (ax.o2 == -1 ? win(3 + j) : win(2 + j));
      const float n3 = ax.o3 == 2 ? win(6 + j) : (ax.o3 == 1 ? win(5 + j) : win(3 + j));
      const float x2 = ax.k2 * n2, x3 = ax.k3 * n3;
      const float y2 = ay.k2 * f4c(y2v, j), y3 = ay.k3 * f4c(y3v, j);
      const float z2 = az.k2 * f4c(z2v, j), z3 = az.k3 * f4c(z3v, j);
      float s = __fmaf_rn(__fadd_rn(__fadd_rn(ax.w, ay.w), az.w), f4c(mid, j), x2);
      s = __fadd_rn(s, x3);
      s = __fadd_rn(s, y2);
      s = __fadd_rn(s, y3);
      s = __fadd_rn(s, z2);
      a[j] = __fadd_rn(s, z3);
    }
    *reinterpret_cast<float4*>(q + base + t) = make_float4(a[0], a[1], a[2], a[3]);
    c = make_float4(__fmul_rn(mid.x, a[0]), __fmul_rn(mid.y, a[1]), __fmul_rn(mid.z, a[2]), __fmul_rn(mid.w, a[3]));
  }
  const float s = block_tree4(c, cc);
  if (threadIdx.x == 0) part[(uint64_t)b * nblk + blockIdx.x] = s;
}

// Final reduction of a solve's block partials (Reduction_lattice,
// Gratings.cu:22-75), then the scalar step: kind 0 -> alpha = delta_new /
// (d . q); kind 1 -> delta_old = delta_new, delta_new = r . r,
// beta = delta_new / delta_old, next step taken while iters < max and
// delta_new > term; kind 2 -> delta_new = r . d at the start.
__global__ void __launch_bounds__(kBlock) svl_reduce_kernel(const float* __restrict__ part, CgState* st, uint32_t nblk,
                                                            uint32_t kind, uint32_t max_iter) {
  __shared__ float cc[kTreeSmem];
  const uint32_t b = blockIdx.x;
  if (kind != 2 && !st[b].active) return;
  const float* pb = part + (uint64_t)b * nblk;
  float c = 0.0f;
  for (uint32_t k = 0; k * kBlock + threadIdx.x < nblk; ++k) c = __fadd_rn(c, pb[k * kBlock + threadIdx.x]);
  const float s = block_tree(c, cc);
  if (threadIdx.x != 0) return;
  CgState& S = st[b];
  if (kind == 0) {
    S.alpha = __fdiv_rn(S.delta_new, s);
  } else if (kind == 1) {
    S.delta_old = S.delta_new;
    S.delta_new = s;
    S.beta = __fdiv_rn(S.delta_new, S.delta_old);
    S.iters += 1;
  } else {
    S.delta_new = s;
    S.iters = 1;
  }
}

// x = 1 x + alpha d, r = 1 r + (-alpha) q (VecSMultAddKernel_lattice,
// Gratings.cu:77-97: a1 * V + a2 * W, the first product fused with the sum of
// the second), and the block partials of r . r.
__device__ __forceinline__ float upd_x(float x, float alpha, float d) { return __fmaf_rn(1.0f, x, __fmul_rn(alpha, d)); }
__device__ __forceinline__ float upd_r(float r, float alpha, float q) {
  return __fmaf_rn(1.0f, r, __fmul_rn(-alpha, q));
}

__global__ void __launch_bounds__(kBlock) svl_update_kernel(float* __restrict__ x, float* __restrict__ r,
                                                            const float* __restrict__ d, const float* __restrict__ q,
                                                            float* __restrict__ part, const CgState* st, uint64_t P,
                                                            uint32_t nblk) {
  __shared__ float cc[kTreeSmem];
  const uint32_t b = blockIdx.y;
  if (!st[b].active) return;
  const uint64_t base = (uint64_t)b * P;
  const uint64_t t = (uint64_t)blockIdx.x * kBlock + threadIdx.x;
  const float alpha = st[b].alpha;
  float c = 0.0f;
  if (t < P) {
    x[base + t] = upd_x(x[base + t], alpha, d[base + t]);
    const float rv = upd_r(r[base + t], alpha, q[base + t]);
    r[base + t] = rv;
    c = __fmul_rn(rv, rv);
  }
  const float s = block_tree(c, cc);
  if (threadIdx.x == 0) part[(uint64_t)b * nblk + blockIdx.x] = s;
}

// The same with 16-byte accesses (P a multiple of 4): a block of 256 threads
// covers the reference's 1024-element reduction block, thread i holding
// elements 4i .. 4i+3.  The tree pairs element t with t + s for s = 512 .. 1,
// which is: across the 8 warps (s = 512, 256, 128), across lanes
// (s = 64 .. 4, shuffles) and inside a thread's four (s = 2, 1).
constexpr int kBlock4 = kBlock / 4;

__global__ void __launch_bounds__(kBlock4) svl_update4_kernel(float4* __restrict__ x, float4* __restrict__ r,
                                                              const float4* __restrict__ d,
                                                              const float4* __restrict__ q, float* __restrict__ part,
                                                              const CgState* st, uint64_t P4, uint32_t nblk) {
  __shared__ float4 cc[kBlock4];
  const uint32_t b = blockIdx.y;
  if (!st[b].active) return;
  const uint64_t base = (uint64_t)b * P4;
  const uint64_t t = (uint64_t)blockIdx.x * kBlock4 + threadIdx.x;
  const float alpha = st[b].alpha;
  float4 c = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  if (t < P4) {
    const float4 xv = x[base + t], dv = d[base + t], rv0 = r[base + t], qv = q[base + t];
    x[base + t] = make_float4(upd_x(xv.x, alpha, dv.x), upd_x(xv.y, alpha, dv.y), upd_x(xv.z, alpha, dv.z),
                              upd_x(xv.w, alpha, dv.w));
    const float4 rv = make_float4(upd_r(rv0.x, alpha, qv.x), upd_r(rv0.y, alpha, qv.y), upd_r(rv0.z, alpha, qv.z),
                                  upd_r(rv0.w, alpha, qv.w));
    r[base + t] = rv;
    c = make_float4(__fmul_rn(rv.x, rv.x), __fmul_rn(rv.y, rv.y), __fmul_rn(rv.z, rv.z), __fmul_rn(rv.w, rv.w));
  }
  cc[threadIdx.x] = c;
  __syncthreads();
  if (threadIdx.x >= 32) return;
  const uint32_t lane = threadIdx.x;
  auto add4 = [](float4 u, float4 v) {
    return make_float4(__fadd_rn(u.x, v.x), __fadd_rn(u.y, v.y), __fadd_rn(u.z, v.z), __fadd_rn(u.w, v.w));
  };
  float4 v[8];
#pragma unroll
  for (int w = 0; w < 8; ++w) v[w] = cc[32 * w + lane];
#pragma unroll
  for (int h = 4; h > 0; h >>= 1)
#pragma unroll
    for (int w = 0; w < h; ++w) v[w] = add4(v[w], v[w + h]);
  float4 a = v[0];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float4 o4 = make_float4(__shfl_down_sync(0xffffffffu, a.x, o), __shfl_down_sync(0xffffffffu, a.y, o),
                                  __shfl_down_sync(0xffffffffu, a.z, o), __shfl_down_sync(0xffffffffu, a.w, o));
    a = add4(a, o4);
  }
  if (lane == 0) part[(uint64_t)b * nblk + blockIdx.x] = __fadd_rn(__fadd_rn(a.x, a.z), __fadd_rn(a.y, a.w));
}

// d = beta d + 1 r, and the decision to take another step
// (the while condition of GPUCG_lattice, Gratings.cu:910-969).
__device__ __forceinline__ float dir_d(float beta, float d, float r) { return __fmaf_rn(beta, d, __fmul_rn(1.0f, r)); }

__global__ void __launch_bounds__(256) svl_dir_kernel(float* __restrict__ d, const float* __restrict__ r, CgState* st,
                                                      uint64_t P, uint32_t max_iter) {
  const uint32_t b = blockIdx.y;
  if (!st[b].active) return;
  const uint64_t base = (uint64_t)b * P;
  const float beta = st[b].beta;
  if ((P & 3u) == 0) {
    float4* d4 = reinterpret_cast<float4*>(d + base);
    const float4* r4 = reinterpret_cast<const float4*>(r + base);
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < P / 4; t += (uint64_t)gridDim.x * blockDim.x) {
      const float4 dv = d4[t], rv = r4[t];
      d4[t] = make_float4(dir_d(beta, dv.x, rv.x), dir_d(beta, dv.y, rv.y), dir_d(beta, dv.z, rv.z),
                          dir_d(beta, dv.w, rv.w));
    }
    return;
  }
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < P; t += (uint64_t)gridDim.x * blockDim.x)
    d[base + t] = dir_d(beta, d[base + t], r[base + t]);
}

__global__ void svl_decide_kernel(CgState* st, uint32_t n, uint32_t max_iter, uint32_t* n_active) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n) return;
  CgState& S = st[b];
  if (S.active) {
    S.active = (S.iters < max_iter && S.delta_new > S.term) ? 1u : 0u;
    if (S.active) atomicAdd(n_active, 1u);
  }
}

__global__ void svl_start_kernel(CgState* st, uint32_t n, uint32_t max_iter, float term, uint32_t* n_active) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n) return;
  CgState& S = st[b];
  S.term = term;
  S.active = (S.iters < max_iter && S.delta_new > term) ? 1u : 0u;
  if (S.active) atomicAdd(n_active, 1u);
}

// Block partials of r . d for the starting delta (every solve).
__global__ void __launch_bounds__(kBlock) svl_dot_kernel(const float* __restrict__ a, const float* __restrict__ bv,
                                                         float* __restrict__ part, uint64_t P, uint32_t nblk) {
  __shared__ float cc[kTreeSmem];
  const uint32_t b = blockIdx.y;
  const uint64_t base = (uint64_t)b * P;
  const uint64_t t = (uint64_t)blockIdx.x * kBlock + threadIdx.x;
  const float c = t < P ? __fmul_rn(a[base + t], bv[base + t]) : 0.0f;
  const float s = block_tree(c, cc);
  if (threadIdx.x == 0) part[(uint64_t)b * nblk + blockIdx.x] = s;
}

// Lattice on the 2x grid: svl += Re(c_m exp(i phi_m)) for m = 0 .. n-1 in
// order (grating_kernel + svl_kernel, Gratings.cu:653-752).  phi_m at fine
// sample (u, v, w) is the coarse solution filtered as an unnormalised linear
// texture with clamped addressing at (u/2 + 1/2, v/2 + 1/2, w/2 + 1/2): the
// weights are 0 or 1/2 on each axis.
__global__ void __launch_bounds__(256) svl_accumulate_kernel(const float* __restrict__ x, const float2* __restrict__ coef,
                                                             uint32_t n, int X, int Y, int Z, uint64_t P,
                                                             float* __restrict__ svl) {
  const int FX = 2 * X, FY = 2 * Y, FZ = 2 * Z;
  const uint64_t F = (uint64_t)FX * FY * FZ;
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < F; t += (uint64_t)gridDim.x * blockDim.x) {
    const int u = (int)(t % FX), v = (int)((t / FX) % FY), w = (int)(t / ((uint64_t)FX * FY));
    const int i0 = u >> 1, j0 = v >> 1, k0 = w >> 1;
    const int i1 = min(i0 + (u & 1), X - 1), j1 = min(j0 + (v & 1), Y - 1), k1 = min(k0 + (w & 1), Z - 1);
    const float fx = (u & 1) ? 0.5f : 0.0f, fy = (v & 1) ? 0.5f : 0.0f, fz = (w & 1) ? 0.5f : 0.0f;
    const int o000 = i0 + X * (j0 + Y * k0), o100 = i1 + X * (j0 + Y * k0), o010 = i0 + X * (j1 + Y * k0),
              o110 = i1 + X * (j1 + Y * k0), o001 = i0 + X * (j0 + Y * k1), o101 = i1 + X * (j0 + Y * k1),
              o011 = i0 + X * (j1 + Y * k1), o111 = i1 + X * (j1 + Y * k1);
    float acc = svl[t];
    for (uint32_t m = 0; m < n; ++m) {
      const float* xm = x + (uint64_t)m * P;
      auto lx = [&](int a, int b) { return __fmaf_rn(fx, __fsub_rn(xm[b], xm[a]), xm[a]); };
      const float c00 = lx(o000, o100), c10 = lx(o010, o110), c01 = lx(o001, o101), c11 = lx(o011, o111);
      const float c0 = __fmaf_rn(fy, __fsub_rn(c10, c00), c00), c1 = __fmaf_rn(fy, __fsub_rn(c11, c01), c01);
      const float ph = __fmaf_rn(fz, __fsub_rn(c1, c0), c0);
      const float2 cm = coef[m];
      const float gr = cosf(ph), gi = sinf(ph);
      acc = __fadd_rn(acc, __fmaf_rn(gr, cm.x, -__fmul_rn(gi, cm.y)));
    }
    svl[t] = acc;
  }
}

// Fourier coefficients of a sampled unit cell at the (2 range + 1)^3
// frequencies, in the reference's order: c = (1/N) sum f e^{-2 pi i (ix/Nx +
// jy/Ny + kz/Nz)} in double (what the reference takes from an R2C cuFFT, scaled
// by 1/N and completed by Hermitian symmetry, src/main.cu:3581-3690).
__global__ void __launch_bounds__(256) svl_dft_kernel(const float* __restrict__ f, uint32_t nx, uint32_t ny, uint32_t nz,
                                                      int range, float2* __restrict__ out) {
  __shared__ double sr[256], si[256];
  const Freq q = freq_of(blockIdx.x, range);
  const uint64_t N = (uint64_t)nx * ny * nz;
  double ar = 0.0, ai = 0.0;
  for (uint64_t t = threadIdx.x; t < N; t += blockDim.x) {
    const uint32_t x = (uint32_t)(t % nx), y = (uint32_t)((t / nx) % ny), z = (uint32_t)(t / ((uint64_t)nx * ny));
    // phase in turns, reduced to [0, 1) exactly in integer arithmetic per axis
    const int64_t px = ((int64_t)q.i * x) % (int64_t)nx, py = ((int64_t)q.j * y) % (int64_t)ny,
                  pz = ((int64_t)q.k * z) % (int64_t)nz;
    const double turns = (double)px / nx + (double)py / ny + (double)pz / nz;
    double s, c;
    sincospi(-2.0 * turns, &s, &c);
    const double v = (double)f[t];
    ar += v * c;
    ai += v * s;
  }
  sr[threadIdx.x] = ar;
  si[threadIdx.x] = ai;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      sr[threadIdx.x] += sr[threadIdx.x + s];
      si[threadIdx.x] += si[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = make_float2((float)(sr[0] / (double)N), (float)(si[0] / (double)N));
}

}  // namespace
}  // namespace gcm

using namespace gcm;

extern "C" {

// set_period_kernel (src/lattice_files/Gratings.cu:818-860): the radial
// period sqrt((u + 1)^2 + (v + 1)^2) of the two sample coordinates across the
// rotation axis ('z': x and y, 'y': x and z, else z and y), each coordinate
// (i - mean) * d.  Written in the reference's expression shapes (plain float
// operators, powf, default contraction: (i - mean) * d + 1 is one fused
// multiply-add), so that the values are the reference's own.
__global__ void __launch_bounds__(256) svl_period_kernel(float* __restrict__ out, uint32_t nx, uint32_t ny,
                                                         uint32_t nz, float dx, float dy, float dz, float mean_x,
                                                         float mean_y, float mean_z, char axis) {
  const uint64_t n = (uint64_t)nx * ny * nz, plane = (uint64_t)nx * ny;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const int xx = (int)(i % nx), yy = (int)((i % plane) / nx), zz = (int)(i / plane);
    const float x = (xx - mean_x) * dx;
    const float y = (yy - mean_y) * dy;
    const float z = (zz - mean_z) * dz;
    float period;
    if (axis == 'z') period = sqrtf(powf(x + 1, 2) + powf(y + 1, 2));
    else if (axis == 'y') period = sqrtf(powf(x + 1, 2) + powf(z + 1, 2));
    else period = sqrtf(powf(z + 1, 2) + powf(y + 1, 2));
    out[i] = period;
  }
}

gcm_status gcm_svl_period_field(gcm_ctx* ctx, float* d_period, uint32_t nx, uint32_t ny, uint32_t nz, float dx,
                                float dy, float dz, float mean_x, float mean_y, float mean_z, char axis,
                                gcm_stream stream) {
  if (!ctx) return GCM_ERR_INVALID_ARGUMENT;
  if (!d_period || nx == 0 || ny == 0 || nz == 0)
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_svl_period_field: bad argument");
  if (axis != 'x' && axis != 'y' && axis != 'z')
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_svl_period_field: axis must be 'x', 'y' or 'z'");
  const uint64_t n = (uint64_t)nx * ny * nz;
  svl_period_kernel<<<grid_blocks(ctx, n, 256, 4), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      d_period, nx, ny, nz, dx, dy, dz, mean_x, mean_y, mean_z, axis);
  GCM_CUDA(ctx, cudaGetLastError());
  count_launch(ctx, 1);
  return GCM_OK;
}

gcm_status gcm_svl_coefficients(gcm_ctx* ctx, uint32_t unit_type, uint32_t unit_n, uint32_t range, float* d_coeff,
                                gcm_stream stream) {
  if (!ctx) return GCM_ERR_INVALID_ARGUMENT;
  if (!d_coeff || unit_n < 2 || range > 8 || unit_type > 5)
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_svl_coefficients: bad argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t n = (size_t)unit_n * unit_n * unit_n;
  gcm_status s = ensure_buffer(ctx, &ctx->field_buf, &ctx->field_bytes, n * sizeof(float));
  if (s) return s;
  s = gcm_field_unit_cell(ctx, unit_type, unit_n, unit_n, unit_n, ctx->field_buf, stream);
  if (s) return s;
  const uint32_t w = 2 * range + 1;
  svl_dft_kernel<<<w * w * w, 256, 0, st>>>(ctx->field_buf, unit_n, unit_n, unit_n, (int)range,
                                            reinterpret_cast<float2*>(d_coeff));
  GCM_CUDA(ctx, cudaGetLastError());
  count_launch(ctx, 1);
  return GCM_OK;
}

gcm_status gcm_svl_lattice(gcm_ctx* ctx, const gcm_svl_params* prm, const float* d_period, const float* d_coeff,
                           float* d_svl, float* d_phase, uint32_t* h_iters, gcm_stream stream) {
  if (!ctx) return GCM_ERR_INVALID_ARGUMENT;
  if (!prm || !d_coeff || !d_svl) return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_svl_lattice: NULL argument");
  const gcm_svl_params& p = *prm;
  if (p.nx < 4 || p.ny < 4 || p.nz < 4)
    return fail(ctx, GCM_ERR_NOT_SUPPORTED, "gcm_svl_lattice: the solve grid needs at least 4 samples per axis");
  const uint32_t w = 2 * p.range + 1;
  if (p.range > 8 || p.n_coeff == 0 || p.n_coeff > w * w * w || p.max_iter == 0)
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_svl_lattice: bad range, coefficient count or iteration cap");
  if (p.period_type > 2 || (p.period_type == 2 && !d_period))
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_svl_lattice: period type 2 needs d_period");
  if (p.kind != 'n' && p.kind != 'r' && p.kind != 'b' && p.kind != 's')
    return fail(ctx, GCM_ERR_INVALID_ARGUMENT, "gcm_svl_lattice: unknown grating kind");
  const uint64_t P = (uint64_t)p.nx * p.ny * p.nz;
  if (P >= (1ull << 31) || 8 * P >= (1ull << 40))
    return fail(ctx, GCM_ERR_NOT_SUPPORTED, "gcm_svl_lattice: grid too large");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const uint32_t B = p.n_coeff;
  const uint32_t nblk = (uint32_t)((P + kBlock - 1) / kBlock);
  // device state: x (phases), r, d, q, partials, per-solve scalars, active count
  float *x = nullptr, *r = nullptr, *dd = nullptr, *q = nullptr, *part = nullptr;
  CgState* cs = nullptr;
  uint32_t* n_active = nullptr;
  const size_t vec = sizeof(float) * P * B;
  auto cleanup = [&] {
    cudaFree(x); cudaFree(r); cudaFree(dd); cudaFree(q); cudaFree(part); cudaFree(cs); cudaFree(n_active);
  };
  if (cudaMalloc(&x, vec) != cudaSuccess || cudaMalloc(&r, vec) != cudaSuccess || cudaMalloc(&dd, vec) != cudaSuccess ||
      cudaMalloc(&q, vec) != cudaSuccess || cudaMalloc(&part, sizeof(float) * (size_t)nblk * B) != cudaSuccess ||
      cudaMalloc(&cs, sizeof(CgState) * B) != cudaSuccess || cudaMalloc(&n_active, sizeof(uint32_t)) != cudaSuccess) {
    cleanup();
    return fail(ctx, GCM_ERR_OUT_OF_MEMORY, "gcm_svl_lattice: %zu bytes of solver state", 4 * vec);
  }
  SvlGeo g{(int)p.nx, (int)p.ny, (int)p.nz, p.dx, p.dy, p.dz, p.kind, p.period_type, p.period, p.period_x,
           p.period_y, p.period_z, p.lcon, p.lcon_1, p.sinewave_z};
  cudaError_t e = cudaMemsetAsync(cs, 0, sizeof(CgState) * B, st);
  if (e == cudaSuccess) {
    svl_rhs_kernel<<<grid_blocks(ctx, P, 256), 256, 0, st>>>(g, d_period, (int)p.range, B, P, x, r, dd);
    e = cudaGetLastError();
  }
  const dim3 gv(nblk, B);
  if (e == cudaSuccess) {
    svl_dot_kernel<<<gv, kBlock, 0, st>>>(r, dd, part, P, nblk);
    svl_reduce_kernel<<<B, kBlock, 0, st>>>(part, cs, nblk, 2, p.max_iter);
    e = cudaMemsetAsync(n_active, 0, sizeof(uint32_t), st);
  }
  // the reference's term = EndRes * EndRes in float
  volatile float er = p.end_res;
  const float term = er * er;
  if (e == cudaSuccess) {
    svl_start_kernel<<<(B + 127) / 128, 128, 0, st>>>(cs, B, p.max_iter, term, n_active);
    e = cudaGetLastError();
  }
  count_launch(ctx, 4);
  // one CG step for every active solve, recorded once and replayed
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t cap = nullptr;
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    cudaMemsetAsync(n_active, 0, sizeof(uint32_t), cap);
    if ((p.nx & 3u) == 0)
      svl_matvec4_kernel<<<gv, kBlock / 4, 0, cap>>>(dd, q, part, cs, g.nx, g.ny, g.nz, make_fastdiv(p.nx),
                                                     make_fastdiv(p.nx * p.ny), P, nblk);
    else
      svl_matvec_kernel<<<gv, kBlock, 0, cap>>>(dd, q, part, cs, g.nx, g.ny, g.nz, make_fastdiv(p.nx),
                                                make_fastdiv(p.nx * p.ny), P, nblk);
    svl_reduce_kernel<<<B, kBlock, 0, cap>>>(part, cs, nblk, 0, p.max_iter);
    if ((P & 3u) == 0)
      svl_update4_kernel<<<gv, kBlock4, 0, cap>>>(reinterpret_cast<float4*>(x), reinterpret_cast<float4*>(r),
                                                 reinterpret_cast<const float4*>(dd),
                                                 reinterpret_cast<const float4*>(q), part, cs, P / 4, nblk);
    else
      svl_update_kernel<<<gv, kBlock, 0, cap>>>(x, r, dd, q, part, cs, P, nblk);
    svl_reduce_kernel<<<B, kBlock, 0, cap>>>(part, cs, nblk, 1, p.max_iter);
    svl_dir_kernel<<<dim3(grid_blocks(ctx, P, 256, 4), B), 256, 0, cap>>>(dd, r, cs, P, p.max_iter);
    svl_decide_kernel<<<(B + 127) / 128, 128, 0, cap>>>(cs, B, p.max_iter, n_active);
    e = cudaStreamEndCapture(cap, &graph);
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
  // replay in bursts; between bursts read how many solves are still running
  uint32_t h_active = 0;
  cudaEvent_t ev = nullptr;
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
  uint32_t steps = 0;
  const uint32_t burst = 16;
  while (e == cudaSuccess && steps + 1 < p.max_iter) {
    // the start kernel's count is the first check
    e = cudaMemcpyAsync(&h_active, n_active, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess || h_active == 0) break;
    if (e == cudaSuccess) e = cudaEventRecord(ev, st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(cap, ev, 0);
    for (uint32_t k = 0; k < burst && e == cudaSuccess && steps + 1 < p.max_iter; ++k, ++steps) {
      e = cudaGraphLaunch(exec, cap);
      count_launch(ctx, 6);
    }
    if (e == cudaSuccess) e = cudaEventRecord(ev, cap);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(st, ev, 0);
  }
  if (e == cudaSuccess) {
    svl_accumulate_kernel<<<grid_blocks(ctx, 8 * P, 256, 8), 256, 0, st>>>(
        x, reinterpret_cast<const float2*>(d_coeff), B, g.nx, g.ny, g.nz, P, d_svl);
    e = cudaGetLastError();
    count_launch(ctx, 1);
  }
  if (e == cudaSuccess && d_phase) e = cudaMemcpyAsync(d_phase, x, vec, cudaMemcpyDeviceToDevice, st);
  std::vector<CgState> hs(B);
  if (e == cudaSuccess) e = cudaMemcpyAsync(hs.data(), cs, sizeof(CgState) * B, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess && h_iters)
    for (uint32_t b = 0; b < B; ++b) h_iters[b] = hs[b].iters;
  if (ev) cudaEventDestroy(ev);
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  if (cap) cudaStreamDestroy(cap);
  cleanup();
  if (e != cudaSuccess) return cuda_fail(ctx, e, "gcm_svl_lattice");
  return GCM_OK;
}

}  // extern "C"
