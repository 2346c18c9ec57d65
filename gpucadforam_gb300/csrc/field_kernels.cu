// Field evaluation kernels for sm_103a: TPMS unit cell, graded TPMS lattices,
// primitive CSG scenes and the band normalisation.
//
// Operation order follows the reference's expressions and is written with
// explicit IEEE intrinsics, so the only difference from a correctly rounded
// evaluation is the accuracy of the CUDA trig functions.
#include <cuda_runtime.h>

#include <algorithm>
#include <float.h>
#include <math.h>
#include <stdint.h>

#include "angle_table.h"
#include "gcm_device.cuh"
#include "gcm_kernels.h"

namespace gcm {

namespace {

__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }

// TPMS from the sines and cosines of the phase (X, Y, Z).  Types: 0 gyroid,
// 1 Schwarz-P, 2 FRD, 3 IWP, 5 Schwarz-D (diamond), after
// src/lattice_files/Fft_lattice.cu:59-85.
__device__ __forceinline__ float tpms_sc(uint32_t type, float sX, float cX, float sY, float cY, float sZ, float cZ) {
  if (type != 2 && type != 3) {
    // gyroid, Schwarz-P and diamond (every other type) each with its own
    // arithmetic, chosen without a branch
    const float gy = fa(fa(fm(sX, cY), fm(sY, cZ)), fm(sZ, cX));
    const float pp = fa(fa(cX, cY), cZ);
    const float dd = fs(fm(fm(cX, cY), cZ), fm(fm(sX, sY), sZ));
    return type == 0 ? gy : (type == 1 ? pp : dd);
  }
  switch (type) {
    case 0: return fa(fa(fm(sX, cY), fm(sY, cZ)), fm(sZ, cX));
    case 1: return fa(fa(cX, cY), cZ);
    case 2: {
      const float c2X = fs(fm(fm(2.0f, cX), cX), 1.0f), c2Y = fs(fm(fm(2.0f, cY), cY), 1.0f),
                  c2Z = fs(fm(fm(2.0f, cZ), cZ), 1.0f);
      return fs(fm(4.0f, fm(fm(cX, cY), cZ)), fa(fa(fm(c2X, c2Y), fm(c2Y, c2Z)), fm(c2Z, c2X)));
    }
    case 3: {
      const float c2X = fs(fm(fm(2.0f, cX), cX), 1.0f), c2Y = fs(fm(fm(2.0f, cY), cY), 1.0f),
                  c2Z = fs(fm(fm(2.0f, cZ), cZ), 1.0f);
      return fs(fm(2.0f, fa(fa(fm(cX, cY), fm(cY, cZ)), fm(cZ, cX))), fa(fa(c2X, c2Y), c2Z));
    }
    default: return fs(fm(fm(cX, cY), cZ), fm(fm(sX, sY), sZ));
  }
}

// ---------------------------------------------------------------------------
// Compensated FP32 arithmetic of the graded lattices.  The phase X of a 512^3
// lattice reaches ~55 half-turns, where one float ulp is 4e-6 half-turns; so
// the parameters, 2/period, the sines and cosines of the Euler angles, the
// rotation and the phase are carried as pairs of floats (hi + lo, ~40 bits)
// and X is reduced mod 2 before its own sin/cos.  Every step is an IEEE float
// add, sub, mul, fma or div in a fixed order (explicit intrinsics, nothing
// contracted), with double add/mul/div/rint only for angles outside
// [-3.156, 3.156]; a CPU restatement of the same sequence gives the same bits.
// ---------------------------------------------------------------------------
struct PF {
  float h, l;
};

__device__ __forceinline__ float fmaf_(float a, float b, float c) { return __fmaf_rn(a, b, c); }

// s + e = a + b exactly (Knuth's branch-free two-sum).
__device__ __forceinline__ PF two_sum(float a, float b) {
  const float s = fa(a, b), bb = fs(s, a);
  return {s, fa(fs(a, fs(s, bb)), fs(b, bb))};
}
__device__ __forceinline__ PF pf_diff(PF b, PF a) {
  const PF d = two_sum(b.h, -a.h);
  return {d.h, fa(d.l, fs(b.l, a.l))};
}
// u + t * d
__device__ __forceinline__ PF pf_at(PF u, PF d, float t) {
  const float p = fm(t, d.h);
  float pe = fmaf_(t, d.h, -p);
  pe = fmaf_(t, d.l, pe);
  const PF s = two_sum(u.h, p);
  return {s.h, fa(fa(s.l, pe), u.l)};
}
__device__ __forceinline__ PF pf_lerp(PF a, PF b, float t) { return pf_at(a, pf_diff(b, a), t); }
__device__ __forceinline__ PF pf_mulf(PF a, float f) {
  const float p = fm(a.h, f);
  float pe = fmaf_(a.h, f, -p);
  pe = fmaf_(a.l, f, pe);
  return {p, pe};
}
__device__ __forceinline__ PF pf_mul(PF a, PF b) {
  const float p = fm(a.h, b.h);
  float pe = fmaf_(a.h, b.h, -p);
  pe = fmaf_(a.h, b.l, pe);
  pe = fmaf_(a.l, b.h, pe);
  return {p, pe};
}
__device__ __forceinline__ PF pf_add(PF a, PF b) {
  const PF s = two_sum(a.h, b.h);
  return {s.h, fa(s.l, fa(a.l, b.l))};
}
__device__ __forceinline__ PF pf_neg(PF a) { return {-a.h, -a.l}; }
// 2 / P: the correctly rounded quotient and its remainder term
__device__ __forceinline__ PF pf_two_over(PF P) {
  const float hh = __fdiv_rn(2.0f, P.h);
  float r = fmaf_(-hh, P.h, 2.0f);
  r = fmaf_(-hh, P.l, r);
  return {hh, fm(r, fm(0.5f, hh))};
}

constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23: adding it rounds to an integer
constexpr uint32_t kAngleRows = 2 * GCM_ANGLE_K + 1;

// sin and cos of an angle pair: the table's sin/cos(k/32) pair nearest the
// angle, corrected by the Taylor series of the remainder d (|d| <= 1/64, terms
// to d^4), renormalised so that later products drop only lo * lo terms.
constexpr float kAngleMax = (float)GCM_ANGLE_K / GCM_ANGLE_STEP_INV;  // the table's reach

__device__ __forceinline__ bool angle_in_table(PF a) { return fabsf(a.h) <= kAngleMax; }

// Angles beyond the table (rare): reduced by 2 pi in double (NaN and
// infinities stay NaN).
__device__ __noinline__ PF reduce_angle(PF a) {
  const double two_pi = 6.283185307179586;
  double A = __dadd_rn((double)a.h, (double)a.l);
  const double m = rint(__ddiv_rn(A, two_pi));
  A = __dsub_rn(A, __dmul_rn(m, two_pi));
  const float h = __double2float_rn(A);
  return {h, __double2float_rn(__dsub_rn(A, (double)h))};
}

// Table part of pf_sincos, for an angle within the table's reach.
__device__ __forceinline__ void pf_sincos_table(PF a, const float4* __restrict__ tab, PF& s, PF& c) {
  const float t = fmaf_(a.h, (float)GCM_ANGLE_STEP_INV, kMagic);
  const float kf = fs(t, kMagic);
  const int k = min(max(__float_as_int(t) - __float_as_int(kMagic), -GCM_ANGLE_K), GCM_ANGLE_K);
  float d = fmaf_(kf, -1.0f / GCM_ANGLE_STEP_INV, a.h);
  d = fa(d, a.l);
  const float4 e = tab[k + GCM_ANGLE_K];
  const float d2 = fm(d, d), d3 = fm(d2, d);
  const float sd = fmaf_(d3, -0x1.555556p-3f, d);
  const float cm1 = fm(d2, fmaf_(d2, 0x1.555556p-5f, -0.5f));
  float sl = fmaf_(e.x, cm1, e.y);
  sl = fmaf_(e.z, sd, sl);
  sl = fmaf_(e.w, sd, sl);
  float cl = fmaf_(e.z, cm1, e.w);
  cl = fmaf_(-e.x, sd, cl);
  cl = fmaf_(-e.y, sd, cl);
  s = two_sum(e.x, sl);
  c = two_sum(e.z, cl);
}

__device__ __forceinline__ void pf_sincos(PF a, const float4* __restrict__ tab, PF& s, PF& c) {
  if (!angle_in_table(a)) a = reduce_angle(a);
  pf_sincos_table(a, tab, s, c);
}

// X mod 2 (half-turns) as one float.
__device__ __forceinline__ float pf_reduce(PF X) {
  const float t = fmaf_(X.h, 0.5f, kMagic);
  const float kf = fs(t, kMagic);
  return fa(fmaf_(kf, -2.0f, X.h), X.l);
}

// sin(pi r), cos(pi r): quarter turn j = rint(2r), u = r - j/2 (|u| <= 1/4),
// Taylor polynomials of sin(pi u) to u^9 and cos(pi u) to u^10.
__device__ __forceinline__ void sincospi_taylor(float r, float& s, float& c) {
  const float t = fmaf_(r, 2.0f, kMagic);
  const float jf = fs(t, kMagic);
  const int j = __float_as_int(t) & 3;
  const float u = fmaf_(jf, -0.5f, r);
  const float z = fm(u, u);
  float ps = fmaf_(z, GCM_SINPI_C9, GCM_SINPI_C7);
  ps = fmaf_(z, ps, GCM_SINPI_C5);
  ps = fmaf_(z, ps, GCM_SINPI_C3);
  ps = fmaf_(z, ps, GCM_SINPI_C1);
  const float sn = fm(u, ps);
  float pc = fmaf_(z, GCM_COSPI_C10, GCM_COSPI_C8);
  pc = fmaf_(z, pc, GCM_COSPI_C6);
  pc = fmaf_(z, pc, GCM_COSPI_C4);
  pc = fmaf_(z, pc, GCM_COSPI_C2);
  const float cs = fmaf_(z, pc, 1.0f);
  // quarter turns: (s, c) = (sn, cs), (cs, -sn), (-sn, -cs), (-cs, sn); the
  // negations as sign-bit flips
  const bool swap = (j & 1) != 0;
  const float a = swap ? cs : sn, b = swap ? sn : cs;
  s = __int_as_float(__float_as_int(a) ^ ((j & 2) << 30));
  c = __int_as_float(__float_as_int(b) ^ (((j + 1) & 2) << 30));
}

__device__ __forceinline__ float tpms_of_phase(uint32_t type, const float r[3], float thick) {
  float s[3], c[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) sincospi_taylor(r[k], s[k], c[k]);
  return fs(tpms_sc(type, s[0], c[0], s[1], c[1], s[2], c[2]), thick);
}

// PARAMS phase: q rotated about x, then y, then z (the rows of Modelling.cu:
// 401-407 applied one axis at a time), scaled by 2/P, reduced mod 2.
__device__ __forceinline__ void params_phase(PF P, PF ax, PF ay, PF az, const float q[3],
                                             const float4* __restrict__ tab, float r[3]) {
  PF sx, cx, sy, cy, sz, cz;
  if (!(angle_in_table(ax) && angle_in_table(ay) && angle_in_table(az))) {  // false for NaN too
    if (!angle_in_table(ax)) ax = reduce_angle(ax);
    if (!angle_in_table(ay)) ay = reduce_angle(ay);
    if (!angle_in_table(az)) az = reduce_angle(az);
  }
  pf_sincos_table(ax, tab, sx, cx);
  pf_sincos_table(ay, tab, sy, cy);
  pf_sincos_table(az, tab, sz, cz);
  const PF v1 = pf_add(pf_mulf(cx, q[1]), pf_neg(pf_mulf(sx, q[2])));
  const PF v2 = pf_add(pf_mulf(sx, q[1]), pf_mulf(cx, q[2]));
  const PF w0 = pf_add(pf_mulf(cy, q[0]), pf_mul(sy, v2));
  const PF w2 = pf_add(pf_mul(cy, v2), pf_neg(pf_mulf(sy, q[0])));
  const PF X0 = pf_add(pf_mul(cz, w0), pf_neg(pf_mul(sz, v1)));
  const PF X1 = pf_add(pf_mul(sz, w0), pf_mul(cz, v1));
  const PF H = pf_two_over(P);
  r[0] = pf_reduce(pf_mul(X0, H));
  r[1] = pf_reduce(pf_mul(X1, H));
  r[2] = pf_reduce(pf_mul(w2, H));
}

// The angle table, copied into shared memory by every graded-lattice CTA.
__device__ const float4 kAngleTable[kAngleRows] = {GCM_ANGLE_TABLE_ROWS};

__device__ __forceinline__ void load_angle_table(float4* s_tab) {
  for (uint32_t i = threadIdx.x; i < kAngleRows; i += blockDim.x) s_tab[i] = kAngleTable[i];
}

// Control-grid cell of one sample coordinate along one axis: the cell index
// i0 (clamped so that i0 + 1 exists), the FP32 fraction inside it, and the
// nearest control point.  Made in FP32 by the kernels and the oracle alike.
struct AxisCell {
  int i0, i1, nearest;
  float f;
};

__device__ __forceinline__ AxisCell locate1(uint32_t pt, uint32_t c, float s) {
  AxisCell k;
  const float cu = fm((float)pt, s);
  int i0 = (int)cu;
  if (c == 1) i0 = 0;
  else if (i0 > (int)c - 2) i0 = (int)c - 2;
  k.i0 = i0;
  k.i1 = c > 1 ? i0 + 1 : 0;
  k.f = c == 1 ? 0.0f : fs(cu, (float)i0);
  int nn = (int)fa(cu, 0.5f);
  if (nn > (int)c - 1) nn = (int)c - 1;
  k.nearest = nn;
  return k;
}

__device__ __forceinline__ uint32_t cidx(int x, int y, int z, const uint32_t c[3]) {
  return (uint32_t)x + c[0] * ((uint32_t)y + c[1] * (uint32_t)z);
}

__device__ __forceinline__ float lerpf(float u, float v, float t) { return __fmaf_rn(t, fs(v, u), u); }

// Trilinear interpolation is evaluated y first, then z, then x:
//   a(xc) = lerp(lerp(v[xc,y0,z0], v[xc,y1,z0], fy), lerp(v[xc,y0,z1], v[xc,y1,z1], fy), fz)
//   value = lerp(a(x0), a(x1), fx)
// so that a(xc) is one number per control column for a whole sample row.
__device__ __forceinline__ float column_yz(const float* __restrict__ a, int xc, const AxisCell& ky,
                                           const AxisCell& kz, const uint32_t c[3]) {
  if (!a) return 0.0f;
  return lerpf(lerpf(__ldg(a + cidx(xc, ky.i0, kz.i0, c)), __ldg(a + cidx(xc, ky.i1, kz.i0, c)), ky.f),
               lerpf(__ldg(a + cidx(xc, ky.i0, kz.i1, c)), __ldg(a + cidx(xc, ky.i1, kz.i1, c)), ky.f), kz.f);
}

// Trilinear weight of corner offset d along one axis.
__device__ __forceinline__ float axis_weight(const AxisCell& k, uint32_t c, int d) {
  if (c == 1) return d ? 0.0f : 1.0f;
  return d ? k.f : fs(1.0f, k.f);
}

}  // namespace

// ---------------------------------------------------------------------------
// create_lattice_kernel (src/lattice_files/Fft_lattice.cu:11-93): the unit-cell
// coordinate is formed in double and rounded to float, the products with the
// literal 3.14 are double and rounded to float at the trig call, type 5 takes
// its first factor through the double cos, type 4 sums double squares.
// ---------------------------------------------------------------------------
//
// Every double operation and every trig call depends on one axis only, so it
// runs once per column (x, per thread) or once per row (y and z, in shared
// memory), not per sample: a sample is then a few float products and one
// store, with the same values.  A CTA takes items of W columns x kUnitRows
// rows (W = nx rounded up to 32, at most 256), 256 / W rows at a time; the
// grid is a multiple of the column chunks, so a CTA keeps one chunk and forms
// its column factors once.
constexpr uint32_t kUnitRows = 64;

namespace {

// The per-axis factors of one TPMS type: t0, t1 floats, d the double cos of
// type 5 (x axis only).
struct UnitAxis {
  float t0, t1;
  double d;
};

__device__ __forceinline__ UnitAxis unit_axis(uint32_t type, uint32_t i, uint32_t n, bool want_double) {
  const float v = (float)(((i * 1.0) / (double)(n - 1) - 0.5) / 0.5);
  const float a = (float)(3.14 * v);
  UnitAxis u{0.0f, 0.0f, 0.0};
  switch (type) {
    case 0: u.t0 = cosf(a); u.t1 = sinf(a); break;
    case 1: u.t0 = cosf(a); break;
    case 2: u.t0 = cosf(v); u.t1 = cosf(fm(2.0f, v)); break;
    case 3: u.t0 = cosf(a); u.t1 = cosf((float)(2 * 3.14 * v)); break;
    case 4: u.t0 = v; break;
    case 5:
      u.t0 = cosf(a);
      u.t1 = sinf(a);
      if (want_double) u.d = cos(3.14 * v);
      break;
    default: break;
  }
  return u;
}

__device__ __forceinline__ float unit_value(uint32_t type, const UnitAxis& X, float y0, float y1, float z0,
                                            float z1) {
  switch (type) {
    case 0: return fa(fa(fm(X.t0, y1), fm(y0, z1)), fm(z0, X.t1));
    case 1: return fa(fa(X.t0, y0), z0);
    case 2: return fs(fm(4.0f, fm(fm(X.t0, y0), z0)), fa(fa(fm(X.t1, y1), fm(y1, z1)), fm(z1, X.t1)));
    case 3: return fs(fm(2.0f, fa(fa(fm(X.t0, y0), fm(y0, z0)), fm(z0, X.t0))), fa(fa(X.t1, y1), z1));
    case 4: {
      const double x2 = (double)fm(X.t0, X.t0), y2 = (double)y0 * (double)y0, z2 = (double)z0 * (double)z0;
      const double xd2 = (double)X.t0 * (double)X.t0;
      return (float)fmin(fmin(x2 + y2, y2 + z2), z2 + xd2);
    }
    case 5: {
      // cos(3.14 x) is the double cos, so the product runs in double left to right
      const double prod = X.d * (double)y0 * (double)z0;
      const float sss = fm(fm(X.t1, y1), z1);
      return (float)(prod - (double)sss);
    }
    default: return 0.0f;
  }
}

}  // namespace

__host__ __device__ inline uint32_t unit_cell_width(uint32_t nx) { return nx >= 256 ? 256 : (nx + 31) & ~31u; }

__global__ void __launch_bounds__(256) unit_cell_kernel(uint32_t type, uint32_t nx, uint32_t ny, uint32_t nz,
                                                        float* out) {
  __shared__ float4 s_row[kUnitRows];  // per row of the item: y factors, z factors
  const uint32_t W = unit_cell_width(nx);
  const uint32_t RS = 256 / W;  // rows in flight
  const uint32_t xl = threadIdx.x % W, rsub = threadIdx.x / W;
  const uint64_t rows = (uint64_t)ny * nz;
  const uint64_t xchunks = (nx + W - 1) / W, rgroups = (rows + kUnitRows - 1) / kUnitRows;
  const uint64_t items = xchunks * rgroups;
  // gridDim.x is a multiple of xchunks: the CTA's column chunk never changes
  const uint32_t x = (uint32_t)(blockIdx.x % xchunks) * W + xl;
  const bool has_x = rsub < RS && x < nx;
  const UnitAxis X = unit_axis(type, has_x ? x : 0, nx, true);
  for (uint64_t it = blockIdx.x; it < items; it += gridDim.x) {
    const uint64_t row0 = (it / xchunks) * kUnitRows;
    const uint32_t nr = rows - row0 < kUnitRows ? (uint32_t)(rows - row0) : kUnitRows;
    __syncthreads();  // the previous item's rows are read
    if (threadIdx.x < nr) {
      const uint64_t row = row0 + threadIdx.x;
      const UnitAxis Y = unit_axis(type, (uint32_t)(row % ny), ny, false);
      const UnitAxis Z = unit_axis(type, (uint32_t)(row / ny), nz, false);
      s_row[threadIdx.x] = make_float4(Y.t0, Y.t1, Z.t0, Z.t1);
    }
    __syncthreads();
    if (!has_x) continue;
    float* o = out + row0 * nx + x;
    for (uint32_t r = rsub; r < nr; r += RS) {
      const float4 q = s_row[r];
      o[(uint64_t)r * nx] = unit_value(type, X, q.x, q.y, q.z, q.w);
    }
  }
}

// ---------------------------------------------------------------------------
// Graded lattices.
// ---------------------------------------------------------------------------

// Blend mode setup: per control point M = R * (2 / period) in double from the
// angle table's sin/cos pairs (rotation rows of Modelling.cu:401-407), each
// entry split into a float pair, then thickness and type:
// GCM_BLEND_WORDS = 20 words (M[r][j] hi, lo at 2 (3r + j)).
__global__ void __launch_bounds__(256) lattice_prep_kernel(LatticeParams p, float* blend_out) {
  const uint32_t n = p.cx * p.cy * p.cz;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float ang[3] = {p.euler ? p.euler[i] : 0.0f, p.euler ? p.euler[n + i] : 0.0f,
                          p.euler ? p.euler[2 * n + i] : 0.0f};
    double S[3], C[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      PF s, c;
      pf_sincos({ang[a], 0.0f}, kAngleTable, s, c);
      S[a] = __dadd_rn((double)s.h, (double)s.l);
      C[a] = __dadd_rn((double)c.h, (double)c.l);
    }
    const double sx = S[0], cx = C[0], sy = S[1], cy = C[1], sz = S[2], cz = C[2];
    double R[9];
    R[0] = __dmul_rn(cz, cy);
    R[1] = __dsub_rn(__dmul_rn(__dmul_rn(cz, sy), sx), __dmul_rn(sz, cx));
    R[2] = __dadd_rn(__dmul_rn(__dmul_rn(cz, sy), cx), __dmul_rn(sz, sx));
    R[3] = __dmul_rn(sz, cy);
    R[4] = __dadd_rn(__dmul_rn(__dmul_rn(sz, sy), sx), __dmul_rn(cz, cx));
    R[5] = __dsub_rn(__dmul_rn(__dmul_rn(sz, sy), cx), __dmul_rn(cz, sx));
    R[6] = -sy;
    R[7] = __dmul_rn(cy, sx);
    R[8] = __dmul_rn(cy, cx);
    const double H = __ddiv_rn(2.0, (double)p.period[i]);
    float* o = blend_out + GCM_BLEND_WORDS * (uint64_t)i;
    for (int k = 0; k < 9; ++k) {
      const double m = __dmul_rn(R[k], H);
      const float hi = __double2float_rn(m);
      o[2 * k] = hi;
      o[2 * k + 1] = __double2float_rn(__dsub_rn(m, (double)hi));
    }
    o[18] = p.thickness ? p.thickness[i] : 0.0f;
    o[19] = __uint_as_float((uint32_t)p.type[i]);
  }
}

// Sample rows are the unit of work.  PARAMS mode: a warp takes R consecutive
// sample rows (y, z) and stages, per control cell i of each row, one 80-byte
// record in its own slice of shared memory (warp syncs only): for period and
// the three Euler angles the y/z-interpolated value at column i and its
// difference to column i + 1 as float pairs, then thickness (value and
// difference) and the types of both columns.  A sample reads its cell's
// record with five 16-byte loads and finishes each parameter with one
// compensated step u + fx * d.  Each lane evaluates two samples of a row (x
// and x + 32) per step.  One row group per warp and many CTAs rather than a
// persistent grid: the block scheduler balances the SMs.
constexpr uint32_t kBlendCx = 128;        // control columns staged per row (BLEND)
constexpr uint32_t kRowWarps = 8;         // warps per CTA of lattice_rows_kernel
constexpr size_t kRowSmem = 48 * 1024;    // shared memory of one such CTA, at most
// control grids too wide for that: one row per warp in opt-in shared memory,
// up to this much per CTA (about 250 control columns)
constexpr size_t kRowSmemWide = 160 * 1024;
constexpr uint32_t kRecWords = 5;         // 16-byte words of one cell record

// Cells of a row: cx - 1 (one for a single control column).
__host__ __device__ constexpr uint32_t row_cells(uint32_t cx) { return cx > 1 ? cx - 1 : 1; }

// 16-byte words of one warp's slice: R rows x (cells + 1) record slots (the
// extra slot holds the last control column while the records are formed), then
// one word per row holding its (y, z) phase coordinates and y, z.
__host__ __device__ constexpr uint32_t row_slots(uint32_t cx) { return row_cells(cx) + 1; }
__host__ __device__ constexpr uint32_t row_slice_words(uint32_t R, uint32_t cx) {
  return R * row_slots(cx) * kRecWords + R;
}
// dynamic shared memory of lattice_rows_kernel: the angle table, then the slices
__host__ __device__ constexpr size_t row_smem_bytes(uint32_t R, uint32_t cx) {
  return (kAngleRows + (size_t)kRowWarps * row_slice_words(R, cx)) * sizeof(float4);
}

namespace {

// Compensated trilinear interpolation of one control array at column xc of
// the sample row's (y, z) cell, y first, then z: pairs all the way.
__device__ __forceinline__ PF column_pf(const float* __restrict__ a, int xc, const AxisCell& ky, const AxisCell& kz,
                                        const uint32_t c[3]) {
  if (!a) return {0.0f, 0.0f};
  const PF A = pf_lerp({__ldg(a + cidx(xc, ky.i0, kz.i0, c)), 0.0f}, {__ldg(a + cidx(xc, ky.i1, kz.i0, c)), 0.0f},
                       ky.f);
  const PF B = pf_lerp({__ldg(a + cidx(xc, ky.i0, kz.i1, c)), 0.0f}, {__ldg(a + cidx(xc, ky.i1, kz.i1, c)), 0.0f},
                       ky.f);
  return pf_lerp(A, B, kz.f);
}

// Staging of one warp's rows, in two passes over all (row, column) pairs so
// that every lane has work.  Pass 1 writes, in slot col of row r, the
// y/z-interpolated values of control column col (the four float pairs, the
// thickness) and its type; pass 2 turns slot i into the record of cell i by
// adding the differences to slot i + 1 (a single column is its own second
// column).  The records are those of one cell at a time: u, v - u.
__device__ __forceinline__ void stage_columns(float4* rec, const float4* sq, uint32_t nr, uint32_t lane,
                                              const float* const arr[5], const uint8_t* __restrict__ type,
                                              const LatticeParams& p, const uint32_t c[3]) {
  const uint32_t cx = c[0], slots = row_slots(cx);
  for (uint32_t j = lane; j < nr * cx; j += 32) {
    const uint32_t r = j / cx, col = j - r * cx;
    const float4 qr = sq[r];
    const AxisCell ky = locate1(__float_as_uint(qr.z), c[1], p.scale[1]);
    const AxisCell kz = locate1(__float_as_uint(qr.w), c[2], p.scale[2]);
    float4* w = rec + (r * slots + col) * kRecWords;
#pragma unroll
    for (uint32_t k = 0; k < 4; ++k) {
      const PF u = column_pf(arr[k], (int)col, ky, kz, c);
      *reinterpret_cast<float2*>(w + k) = make_float2(u.h, u.l);
    }
    w[4].x = column_yz(arr[4], (int)col, ky, kz, c);
    w[4].z = __uint_as_float((uint32_t)__ldg(type + cidx((int)col, ky.nearest, kz.nearest, c)));
  }
  __syncwarp();
  const uint32_t cells = row_cells(cx);
  for (uint32_t j = lane; j < nr * cells; j += 32) {
    const uint32_t r = j / cells, i = j - r * cells;
    float4* w0 = rec + (r * slots + i) * kRecWords;
    const float4* w1 = cx > 1 ? w0 + kRecWords : w0;
#pragma unroll
    for (uint32_t k = 0; k < 4; ++k) {
      const float2 u = *reinterpret_cast<const float2*>(w0 + k), v = *reinterpret_cast<const float2*>(w1 + k);
      const PF d = pf_diff({v.x, v.y}, {u.x, u.y});
      *reinterpret_cast<float2*>(reinterpret_cast<float*>(w0 + k) + 2) = make_float2(d.h, d.l);
    }
    const float tu = w0[4].x, tv = w1[4].x, t1 = w1[4].z;
    w0[4].y = fs(tv, tu);
    w0[4].w = t1;
  }
}

// One staged sample from its cell's record: parameters, phase, TPMS value.
// The nearest control column is the cell's first or second column.
__device__ __forceinline__ float record_sample(const float4* __restrict__ rec, const AxisCell& kx, float qx,
                                               float2 qyz, const float4* __restrict__ tab) {
  const float4* r = rec + kRecWords * kx.i0;
  const float4 a = r[0], b = r[1], c = r[2], d = r[3], e = r[4];
  const float f = kx.f;
  const PF P = pf_at({a.x, a.y}, {a.z, a.w}, f), ex = pf_at({b.x, b.y}, {b.z, b.w}, f),
           ey = pf_at({c.x, c.y}, {c.z, c.w}, f), ez = pf_at({d.x, d.y}, {d.z, d.w}, f);
  const float thick = fmaf_(f, e.y, e.x);
  const uint32_t type = __float_as_uint(kx.nearest == kx.i0 ? e.z : e.w);
  const float q[3] = {qx, qyz.x, qyz.y};
  float rr[3];
  params_phase(P, ex, ey, ez, q, tab, rr);
  return tpms_of_phase(type, rr, thick);
}

// One unstaged sample: the same values as record_sample from the global arrays.
__device__ __forceinline__ float params_sample(const float* const arr[5], const uint8_t* __restrict__ type,
                                               const AxisCell& kx, const AxisCell& ky, const AxisCell& kz,
                                               const uint32_t c[3], const float q[3],
                                               const float4* __restrict__ tab) {
  PF v[4];
#pragma unroll
  for (uint32_t k = 0; k < 4; ++k) {
    const PF u = column_pf(arr[k], kx.i0, ky, kz, c);
    v[k] = pf_at(u, pf_diff(column_pf(arr[k], kx.i1, ky, kz, c), u), kx.f);
  }
  const float tu = column_yz(arr[4], kx.i0, ky, kz, c);
  const float thick = fmaf_(kx.f, fs(column_yz(arr[4], kx.i1, ky, kz, c), tu), tu);
  const uint32_t t = __ldg(type + cidx(kx.nearest, ky.nearest, kz.nearest, c));
  float rr[3];
  params_phase(v[0], v[1], v[2], v[3], q, tab, rr);
  return tpms_of_phase(t, rr, thick);
}

}  // namespace

// CTAs per SM the register budget of lattice_rows_kernel is sized for.
#ifndef GCM_LATTICE_ROWS_MIN_CTAS
#define GCM_LATTICE_ROWS_MIN_CTAS 5
#endif

template <uint32_t R>
__global__ void __launch_bounds__(256, GCM_LATTICE_ROWS_MIN_CTAS) lattice_rows_kernel(LatticeParams p) {
  extern __shared__ float4 s_dyn[];
  float4* s_tab = s_dyn;
  float4* s_rows = s_dyn + kAngleRows;
  load_angle_table(s_tab);
  __syncthreads();
  const uint32_t cx = p.cx;
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  const uint32_t slots = row_slots(cx);
  float4* rec = s_rows + warp * row_slice_words(R, cx);
  float4* sq = rec + R * slots * kRecWords;
  const uint32_t c[3] = {p.cx, p.cy, p.cz};
  const uint32_t nc = p.cx * p.cy * p.cz;
  const float* arr[5] = {p.period, p.euler, p.euler ? p.euler + nc : nullptr,
                         p.euler ? p.euler + 2 * nc : nullptr, p.thickness};
  const uint32_t rows = p.ny * p.nz;
  const uint32_t groups = (rows + R - 1) / R;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t g = blockIdx.x * (blockDim.x >> 5) + warp; g < groups; g += warps) {
    const uint32_t row0 = g * R, nr = min(R, rows - row0);
    __syncwarp();  // the warp's previous group is read
    if (lane < nr) {
      const uint32_t y = (row0 + lane) % p.ny, z = (row0 + lane) / p.ny;
      sq[lane] = make_float4(fs((float)y, p.origin[1]), fs((float)z, p.origin[2]), __uint_as_float(y),
                             __uint_as_float(z));
    }
    __syncwarp();
    stage_columns(rec, sq, nr, lane, arr, p.type, p, c);
    __syncwarp();
    for (uint32_t x0 = lane; x0 < p.nx; x0 += 64) {
      const uint32_t x1 = x0 + 32;
      const AxisCell k0 = locate1(x0, c[0], p.scale[0]);
      const float q0 = fs((float)x0, p.origin[0]);
      float* out = p.out + (uint64_t)row0 * p.nx + x0;
      if (x0 - lane + 32 < p.nx) {  // warp-uniform: the second segment holds samples
        const AxisCell k1 = locate1(min(x1, p.nx - 1), c[0], p.scale[0]);
        const float q1 = fs((float)x1, p.origin[0]);
#pragma unroll 1
        for (uint32_t r = 0; r < nr; ++r) {
          const float4* rr = rec + r * slots * kRecWords;
          const float4 qr = sq[r];
          const float v0 = record_sample(rr, k0, q0, make_float2(qr.x, qr.y), s_tab);
          const float v1 = record_sample(rr, k1, q1, make_float2(qr.x, qr.y), s_tab);
          out[(uint64_t)r * p.nx] = v0;
          if (x1 < p.nx) out[(uint64_t)r * p.nx + 32] = v1;
        }
      } else {
#pragma unroll 1
        for (uint32_t r = 0; r < nr; ++r) {
          const float4 qr = sq[r];
          out[(uint64_t)r * p.nx] = record_sample(rec + r * slots * kRecWords, k0, q0, make_float2(qr.x, qr.y), s_tab);
        }
      }
    }
  }
}

// Control grids too wide for a warp's slice of one row: every sample reads its columns.
__global__ void __launch_bounds__(256) lattice_params_kernel(LatticeParams p) {
  __shared__ float4 s_tab[kAngleRows];
  load_angle_table(s_tab);
  __syncthreads();
  const uint32_t c[3] = {p.cx, p.cy, p.cz};
  const uint32_t nc = p.cx * p.cy * p.cz;
  const float* arr[5] = {p.period, p.euler, p.euler ? p.euler + nc : nullptr,
                         p.euler ? p.euler + 2 * nc : nullptr, p.thickness};
  const uint32_t rows = p.ny * p.nz;
  for (uint32_t row = blockIdx.x; row < rows; row += gridDim.x) {
    const uint32_t y = row % p.ny, z = row / p.ny;
    const AxisCell ky = locate1(y, c[1], p.scale[1]), kz = locate1(z, c[2], p.scale[2]);
    float* out = p.out + (uint64_t)row * p.nx;
    for (uint32_t x = threadIdx.x; x < p.nx; x += blockDim.x) {
      const AxisCell kx = locate1(x, c[0], p.scale[0]);
      const float q[3] = {fs((float)x, p.origin[0]), fs((float)y, p.origin[1]), fs((float)z, p.origin[2])};
      out[x] = params_sample(arr, p.type, kx, ky, kz, c, q, s_tab);
    }
  }
}

namespace {

// BLEND mode: phase of one corner lattice, X_r = M_r0 q0 + K_r with
// K_r = M_r1 q1 + M_r2 q2 (constant along a sample row).
__device__ __forceinline__ PF blend_k(const float* __restrict__ rec, uint32_t r, float q1, float q2) {
  return pf_add(pf_mulf({rec[6 * r + 2], rec[6 * r + 3]}, q1), pf_mulf({rec[6 * r + 4], rec[6 * r + 5]}, q2));
}

}  // namespace

namespace {

// One sample row of the blend form: its control cells along y and z, the
// corner rows' phase coordinates and the y/z part of the trilinear weights.
struct BlendRow {
  AxisCell ky, kz;
  int gy[2], gz[2];
  float qy[2], qz[2], wyz[4];
};

__device__ __forceinline__ BlendRow blend_row(const LatticeParams& p, const uint32_t c[3], uint32_t y, uint32_t z) {
  BlendRow R;
  R.ky = locate1(y, c[1], p.scale[1]);
  R.kz = locate1(z, c[2], p.scale[2]);
  R.gy[0] = c[1] > 1 ? R.ky.i0 : 0;
  R.gy[1] = c[1] > 1 ? R.ky.i0 + 1 : 0;
  R.gz[0] = c[2] > 1 ? R.kz.i0 : 0;
  R.gz[1] = c[2] > 1 ? R.kz.i0 + 1 : 0;
#pragma unroll
  for (int d = 0; d < 2; ++d) {
    R.qy[d] = fs((float)y, c[1] > 1 ? fm((float)R.gy[d], p.anchor[1]) : 0.0f);
    R.qz[d] = fs((float)z, c[2] > 1 ? fm((float)R.gz[d], p.anchor[2]) : 0.0f);
  }
#pragma unroll
  for (int dz = 0; dz < 2; ++dz)
#pragma unroll
    for (int dy = 0; dy < 2; ++dy)
      R.wyz[2 * dz + dy] = fm(axis_weight(R.ky, c[1], dy), axis_weight(R.kz, c[2], dz));
  return R;
}

// The staged record of corner row (dy, dz) = corner and control column xc:
// M_r0 pairs (3), K_r pairs (3), thickness, type.
__device__ __forceinline__ void blend_stage(const LatticeParams& p, const uint32_t c[3], const BlendRow& R,
                                            uint32_t corner, uint32_t xc, float4* w) {
  const int dy = corner & 1, dz = corner >> 1;
  const int gyc = dy ? R.gy[1] : R.gy[0], gzc = dz ? R.gz[1] : R.gz[0];
  const float qyc = dy ? R.qy[1] : R.qy[0], qzc = dz ? R.qz[1] : R.qz[0];
  const float* rec = p.blend + GCM_BLEND_WORDS * (uint64_t)cidx((int)xc, gyc, gzc, c);
  float m[6];
#pragma unroll
  for (uint32_t r = 0; r < 3; ++r) {
    m[2 * r] = __ldg(rec + 6 * r);
    m[2 * r + 1] = __ldg(rec + 6 * r + 1);
  }
  const PF K0 = blend_k(rec, 0, qyc, qzc), K1 = blend_k(rec, 1, qyc, qzc), K2 = blend_k(rec, 2, qyc, qzc);
  w[0] = make_float4(m[0], m[1], m[2], m[3]);
  w[1] = make_float4(m[4], m[5], K0.h, K0.l);
  w[2] = make_float4(K1.h, K1.l, K2.h, K2.l);
  w[3] = make_float4(__ldg(rec + 18), __ldg(rec + 19), 0.0f, 0.0f);
}

// One sample: the weighted sum of the 8 corner lattices.  rec(corner, xc)
// gives the staged record, or null for the unstaged form (read from p.blend).
template <typename Rec>
__device__ __forceinline__ float blend_sample(const LatticeParams& p, const uint32_t c[3], const BlendRow& R,
                                              uint32_t x, Rec rec) {
  const AxisCell kx = locate1(x, c[0], p.scale[0]);
  const int gx[2] = {c[0] > 1 ? kx.i0 : 0, c[0] > 1 ? kx.i0 + 1 : 0};
  float acc = 0.0f;
#pragma unroll 1
  for (int corner = 0; corner < 8; ++corner) {
    // selects rather than run-time array indices keep R in registers
    const int dx = corner & 1, dy = (corner >> 1) & 1, dz = corner >> 2;
    const float wyz = dz ? (dy ? R.wyz[3] : R.wyz[2]) : (dy ? R.wyz[1] : R.wyz[0]);
    const int gxc = dx ? gx[1] : gx[0], gyc = dy ? R.gy[1] : R.gy[0], gzc = dz ? R.gz[1] : R.gz[0];
    const float qyc = dy ? R.qy[1] : R.qy[0], qzc = dz ? R.qz[1] : R.qz[0];
    const float w = fm(axis_weight(kx, c[0], dx), wyz);
    if (w == 0.0f) continue;
    const float q0 = fs((float)x, c[0] > 1 ? fm((float)gxc, p.anchor[0]) : 0.0f);
    PF M0, M1, M2, K0, K1, K2;
    float thick;
    uint32_t type;
    const float4* s = rec(2 * dz + dy, gxc);
    if (s) {
      const float4 a = s[0], b = s[1], e = s[2], f = s[3];
      M0 = {a.x, a.y};
      M1 = {a.z, a.w};
      M2 = {b.x, b.y};
      K0 = {b.z, b.w};
      K1 = {e.x, e.y};
      K2 = {e.z, e.w};
      thick = f.x;
      type = __float_as_uint(f.y);
    } else {
      const float* g = p.blend + GCM_BLEND_WORDS * (uint64_t)cidx(gxc, gyc, gzc, c);
      M0 = {__ldg(g + 0), __ldg(g + 1)};
      M1 = {__ldg(g + 6), __ldg(g + 7)};
      M2 = {__ldg(g + 12), __ldg(g + 13)};
      K0 = blend_k(g, 0, qyc, qzc);
      K1 = blend_k(g, 1, qyc, qzc);
      K2 = blend_k(g, 2, qyc, qzc);
      thick = __ldg(g + 18);
      type = __float_as_uint(__ldg(g + 19));
    }
    const float r[3] = {pf_reduce(pf_add(pf_mulf(M0, q0), K0)), pf_reduce(pf_add(pf_mulf(M1, q0), K1)),
                        pf_reduce(pf_add(pf_mulf(M2, q0), K2))};
    acc = fmaf_(w, tpms_of_phase(type, r, thick), acc);
  }
  return acc;
}

}  // namespace

// BLEND mode, CTA per sample row: the row's records staged by the whole CTA
// (control grids up to kBlendCx columns), else read from the setup buffer.
__global__ void __launch_bounds__(256) lattice_blend_kernel(LatticeParams p) {
  __shared__ float4 s_rec[4][kBlendCx][4];
  const uint32_t c[3] = {p.cx, p.cy, p.cz};
  const bool staged = p.cx <= kBlendCx;
  const uint32_t rows = p.ny * p.nz;
  for (uint32_t row = blockIdx.x; row < rows; row += gridDim.x) {
    const BlendRow R = blend_row(p, c, row % p.ny, row / p.ny);
    if (staged) {
      __syncthreads();  // the previous row's records are read
      for (uint32_t i = threadIdx.x; i < 4 * p.cx; i += blockDim.x)
        blend_stage(p, c, R, i / p.cx, i % p.cx, s_rec[i / p.cx][i % p.cx]);
      __syncthreads();
    }
    float* out = p.out + (uint64_t)row * p.nx;
    for (uint32_t x = threadIdx.x; x < p.nx; x += blockDim.x)
      out[x] = blend_sample(p, c, R, x, [&](int corner, int xc) -> const float4* {
        return staged ? s_rec[corner][xc] : nullptr;
      });
  }
}

// BLEND mode, warp per sample row: each warp stages its row's records in its
// own slice of shared memory (warp syncs only, no CTA barrier) for control
// grids up to kBlendWarpCxWide columns (opt-in shared memory above
// kBlendWarpCx).  Same values as lattice_blend_kernel.
constexpr uint32_t kBlendWarps = 8;
constexpr uint32_t kBlendWarpCx = 24;      // 8 warps x 4 corner rows x 24 columns x 64 B = 48 KB
constexpr uint32_t kBlendWarpCxWide = 80;  // the same in opt-in shared memory: 160 KB

__global__ void __launch_bounds__(kBlendWarps * 32, 6) lattice_blend_warp_kernel(LatticeParams p) {
  extern __shared__ float4 s_blend[];
  const uint32_t c[3] = {p.cx, p.cy, p.cz};
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  float4* rec = s_blend + (size_t)warp * 4u * p.cx * 4u;  // [corner][xc][4]
  const uint32_t rows = p.ny * p.nz;
  const uint32_t nw = gridDim.x * kBlendWarps;
  for (uint32_t row = blockIdx.x * kBlendWarps + warp; row < rows; row += nw) {
    const BlendRow R = blend_row(p, c, row % p.ny, row / p.ny);
    __syncwarp();  // the previous row's records are read
    for (uint32_t i = lane; i < 4 * p.cx; i += 32) blend_stage(p, c, R, i / p.cx, i % p.cx, rec + 4u * i);
    __syncwarp();
    float* out = p.out + (uint64_t)row * p.nx;
    for (uint32_t x = lane; x < p.nx; x += 32)
      out[x] = blend_sample(p, c, R, x, [&](int corner, int xc) -> const float4* {
        return rec + 4u * ((uint32_t)corner * p.cx + (uint32_t)xc);
      });
  }
}

// Batched graded lattices (GCM_GRADE_PARAMS): the sample rows of all
// instances form one sequence of row groups (BatchLattice); a warp takes one
// group at a time.  A staged group holds up to 32 / cx rows of one instance:
// lane (r, col) stages control column col of row r, so every lane has a column
// to interpolate, and the cell records go into the warp's own slice of shared
// memory as in lattice_rows_kernel.  The group's samples are then one run
// (its rows are consecutive in the output), two per lane per step, so short
// rows leave no lanes idle at their ends.  Same values as the single-grid
// kernels.
constexpr uint32_t kWarpCx = GCM_BATCH_WARP_CX;  // control columns staged per warp
constexpr uint32_t kGroupRows = 8;                // rows of a group, at most

// STAGED: the groups of instances with at most kWarpCx control columns (the
// other groups are skipped); the other form takes the wider ones, a row each.
template <bool STAGED>
__global__ void __launch_bounds__(256, 5) lattice_params_batch_kernel(const BatchLattice* inst, uint32_t n_inst,
                                                                   uint64_t total_groups) {
  __shared__ float4 s_rec[8][kRecWords * kWarpCx];  // per warp: the group's cell records
  __shared__ float2 s_q[8][kGroupRows];             // per warp: the (y, z) phase coordinates of each row
  __shared__ float4 s_tab[kAngleRows];
  load_angle_table(s_tab);
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31u, wib = threadIdx.x >> 5;
  const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
  uint32_t lo = 0;  // instance of the warp's group: groups only increase, so search only when it moves on
  for (uint64_t grp = (uint64_t)blockIdx.x * (blockDim.x >> 5) + wib; grp < total_groups; grp += warps) {
    if (lo + 1 < n_inst && inst[lo + 1].group_begin <= grp) {
      uint32_t a = lo + 1, b = n_inst - 1;  // last instance with group_begin <= grp
      while (a < b) {
        const uint32_t mid = (a + b + 1) / 2;
        if (inst[mid].group_begin <= grp) a = mid;
        else b = mid - 1;
      }
      lo = a;
    }
    const LatticeParams& p = inst[lo].p;
    if ((p.cx <= kWarpCx) != STAGED) continue;  // warp-uniform
    const uint32_t R = inst[lo].group_rows;
    const uint32_t rows = p.ny * p.nz;
    const uint32_t row0 = (uint32_t)(grp - inst[lo].group_begin) * R;
    const uint32_t nr = min(R, rows - row0);
    const uint32_t c[3] = {p.cx, p.cy, p.cz};
    const uint32_t nc = p.cx * p.cy * p.cz;
    const float* arr[5] = {p.period, p.euler, p.euler ? p.euler + nc : nullptr,
                           p.euler ? p.euler + 2 * nc : nullptr, p.thickness};
    __syncwarp();  // the warp's previous group is read
    if (STAGED) {
      // lane = r * cx + col; a cell's second column is the next lane's (a
      // single column is its own)
      const uint32_t cells = row_cells(p.cx);
      const uint32_t r = lane / p.cx, col = lane - r * p.cx;
      const bool has_col = r < nr;
      const uint32_t row = row0 + (has_col ? r : 0);
      const uint32_t y = row % p.ny, z = row / p.ny;
      const AxisCell ky = locate1(y, c[1], p.scale[1]), kz = locate1(z, c[2], p.scale[2]);
      PF u[4];
#pragma unroll
      for (uint32_t k = 0; k < 4; ++k) u[k] = column_pf(arr[k], (int)col, ky, kz, c);
      const float tu = column_yz(arr[4], (int)col, ky, kz, c);
      const uint32_t t0 = __ldg(p.type + cidx((int)col, ky.nearest, kz.nearest, c));
      PF v[4];
#pragma unroll
      for (uint32_t k = 0; k < 4; ++k)
        v[k] = {__shfl_down_sync(0xffffffffu, u[k].h, 1), __shfl_down_sync(0xffffffffu, u[k].l, 1)};
      float tv = __shfl_down_sync(0xffffffffu, tu, 1);
      uint32_t t1 = __shfl_down_sync(0xffffffffu, t0, 1);
      if (p.cx == 1) {
#pragma unroll
        for (uint32_t k = 0; k < 4; ++k) v[k] = u[k];
        tv = tu;
        t1 = t0;
      }
      if (has_col && col < cells) {
        float4* w = &s_rec[wib][kRecWords * (r * cells + col)];
#pragma unroll
        for (uint32_t k = 0; k < 4; ++k) {
          const PF d = pf_diff(v[k], u[k]);
          w[k] = make_float4(u[k].h, u[k].l, d.h, d.l);
        }
        w[4] = make_float4(tu, fs(tv, tu), __uint_as_float(t0), __uint_as_float(t1));
      }
      if (has_col && col == 0) s_q[wib][r] = make_float2(fs((float)y, p.origin[1]), fs((float)z, p.origin[2]));
      __syncwarp();
      // the group's samples as one run: sample j is row j / nx, column j % nx
      float* out = p.out + (uint64_t)row0 * p.nx;
      const uint32_t total = nr * p.nx, stride = cells * kRecWords;
      uint32_t ra = 0, xa = lane;  // row and column of sample j = j0 (j0 = lane + 64 k)
      while (xa >= p.nx) {
        xa -= p.nx;
        ++ra;
      }
      for (uint32_t j0 = lane; j0 < total; j0 += 64) {
        uint32_t rb = ra, xb = xa + 32;  // sample j0 + 32
        while (xb >= p.nx) {
          xb -= p.nx;
          ++rb;
        }
        const AxisCell k0 = locate1(xa, c[0], p.scale[0]);
        const float v0 = record_sample(&s_rec[wib][ra * stride], k0, fs((float)xa, p.origin[0]), s_q[wib][ra], s_tab);
        if (j0 + 32 < total) {
          const AxisCell k1 = locate1(xb, c[0], p.scale[0]);
          const float v1 =
              record_sample(&s_rec[wib][rb * stride], k1, fs((float)xb, p.origin[0]), s_q[wib][rb], s_tab);
          out[j0] = v0;
          out[j0 + 32] = v1;
        } else {
          out[j0] = v0;
        }
        xa = xb + 32;  // sample j0 + 64
        ra = rb;
        while (xa >= p.nx) {
          xa -= p.nx;
          ++ra;
        }
      }
    } else {
      for (uint32_t r = 0; r < nr; ++r) {
        const uint32_t row = row0 + r, y = row % p.ny, z = row / p.ny;
        const AxisCell ky = locate1(y, c[1], p.scale[1]), kz = locate1(z, c[2], p.scale[2]);
        float* out = p.out + (uint64_t)row * p.nx;
        for (uint32_t x = lane; x < p.nx; x += 32) {
          const AxisCell kx = locate1(x, c[0], p.scale[0]);
          const float q[3] = {fs((float)x, p.origin[0]), fs((float)y, p.origin[1]), fs((float)z, p.origin[2])};
          out[x] = params_sample(arr, p.type, kx, ky, kz, c, q, s_tab);
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Primitive CSG.  Per primitive, the point-independent parts of the reference
// kernels (rotation rows, normalised cylinder axis, its end point and length)
// are computed once per CTA; they are the same values every reference thread
// computes for itself.
// ---------------------------------------------------------------------------
namespace {

struct PrimPre {
  uint32_t kind, op, flag, pad;
  float c[3];
  float p[6];
  float R[9];      // rotated kinds: rows of the ZYX basis
  float ang[3];    // rotated kinds: the Euler angles
  float sy;        // rotated kinds: sin(angle y)
  float axis[3];   // cylinder: unit axis
  float end[3];    // cylinder: center + axis
  float w3[3];     // cylinder: end - center
  float dis;       // cylinder: |w3|
};

__device__ __forceinline__ float sqf(float x) { return fm(x, x); }

// Per primitive, the sample-independent values every thread of the reference
// kernels computes for itself (src/Modelling.cu:264-270, 401-407).  The basis
// rows are written in the reference's expression shapes (CUDA sinf/cosf,
// plain operators) so that nvcc rounds and contracts them the same way.
// EXACT: the axis length of a cylinder squares with powf as the reference
// does; otherwise with correctly rounded products.
template <bool EXACT>
__device__ void prim_setup(const gcm_primitive& q, PrimPre& o) {
  o.kind = q.kind;
  o.op = q.op;
  o.flag = q.flag;
  for (int a = 0; a < 3; ++a) o.c[a] = q.center[a];
  for (int a = 0; a < 6; ++a) o.p[a] = q.p[a];
  if (q.kind == 1) {
    float am;
    if constexpr (EXACT) am = sqrtf(powf(q.v3[0], 2) + powf(q.v3[1], 2) + powf(q.v3[2], 2));
    else am = __fsqrt_rn(fa(fa(sqf(q.v3[0]), sqf(q.v3[1])), sqf(q.v3[2])));
    for (int a = 0; a < 3; ++a) {
      o.axis[a] = __fdiv_rn(q.v3[a], am);
      o.end[a] = fa(o.axis[a], q.center[a]);
    }
    for (int a = 0; a < 3; ++a) o.w3[a] = fs(o.end[a], q.center[a]);
    if constexpr (EXACT) o.dis = sqrtf(powf(o.w3[0], 2) + powf(o.w3[1], 2) + powf(o.w3[2], 2));
    else o.dis = __fsqrt_rn(fa(fa(sqf(o.w3[0]), sqf(o.w3[1])), sqf(o.w3[2])));
  } else if (q.kind >= 2) {
    const float ax = q.v3[0], ay = q.v3[1], az = q.v3[2];
    o.ang[0] = ax;
    o.ang[1] = ay;
    o.ang[2] = az;
    o.R[0] = cosf(az) * cosf(ay);
    o.R[1] = (cosf(az) * sinf(ay) * sinf(ax)) - (sinf(az) * cosf(ax));
    o.R[2] = (cosf(az) * sinf(ay) * cosf(ax)) + (sinf(az) * sinf(ax));
    o.R[3] = (sinf(az)) * cosf(ay);
    o.R[4] = (sinf(az) * sinf(ay) * sinf(ax)) + (cosf(az) * cosf(ax));
    o.R[5] = (sinf(az) * sinf(ay) * cosf(ax)) - (cosf(az) * sinf(ax));
    o.R[6] = -1.0f * sinf(ay);
    o.R[7] = cosf(ay) * sinf(ax);
    o.R[8] = cosf(ay) * cosf(ax);
    o.sy = sinf(ay);
  }
}

// Field of one primitive of kind K at sample offset t = index - origin (per
// axis) and spacing sp, after the kernels of src/Modelling.cu, with the
// rounding pattern of the reference's own build (nvcc default contraction):
// the position t * sp - c is one fused multiply-add, the sums of products in
// the basis rows, cross products and the cylinder's axial distance fuse their
// first product, 1 - 2 products of a lerp (pyramid widths) fuse, and literals
// such as 2.0 and 100 promote the cone height terms to double.  Every
// operation is an explicit IEEE intrinsic, so the CPU oracle restates it bit
// for bit.  Squares are correctly rounded products; the reference squares
// with powf(v, 2), which differs from the rounded square in the last bit for
// about 6% of floats, so these fields stay within a few ulp of the
// reference's (prim_eval_exact reproduces it bit for bit).  Kinds 7 and
// above are pyramid frustums.
__device__ __forceinline__ void rotate_ref(const PrimPre& P, float x, float y, float z, float& a, float& b,
                                           float& cc) {
  a = __fmaf_rn(z, P.R[2], __fmaf_rn(x, P.R[0], fm(y, P.R[1])));
  b = __fmaf_rn(z, P.R[5], __fmaf_rn(x, P.R[3], fm(y, P.R[4])));
  // the reference's -1.0f * sinf(angle y) folds into y * R7 - x * sin(angle y)
  cc = __fmaf_rn(z, P.R[8], __fmaf_rn(y, P.R[7], -fm(x, P.sy)));
}

// The cone height terms: g = y - h/2 and the slab max((g - h/2)*100,
// -(g + h/2)*100), in double as the reference's literals make them.
__device__ __forceinline__ float cone_slab(float b, float h) {
  const float g = (float)__dsub_rn((double)b, (double)h / 2.0);
  return (float)fmax(__dmul_rn(__dsub_rn((double)g, (double)h / 2.0), 100.0),
                     -__dmul_rn(__dadd_rn((double)g, (double)h / 2.0), 100.0));
}

template <int K>
__device__ __forceinline__ float prim_eval_k(const PrimPre& P, float tx, float ty, float tz, const float sp[3]) {
  if constexpr (K == 0) {  // implicit_sphere_kernel :314-361
    const float x = __fmaf_rn(tx, sp[0], -P.c[0]), y = __fmaf_rn(ty, sp[1], -P.c[1]),
                z = __fmaf_rn(tz, sp[2], -P.c[2]);
    const float r = P.p[0], td = fm(P.p[1], 0.5f);
    const float d2 = fa(fa(sqf(x), sqf(y)), sqf(z));
    if (P.flag) return fmaxf(-fs(d2, sqf(fs(r, td))), fs(d2, sqf(fa(r, td))));
    return fs(d2, sqf(r));
  } else if constexpr (K == 1) {  // distance_from_line_kernel :244-302
    const float r = P.p[0], td = fm(P.p[1], 0.5f), tda = fm(P.p[2], 0.5f);
    float w1[3], w2[3];
    const float t[3] = {tx, ty, tz};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      w1[a] = __fmaf_rn(t[a], sp[a], -P.c[a]);
      w2[a] = __fmaf_rn(t[a], sp[a], -P.end[a]);
    }
    const float dx = __fmaf_rn(w1[1], w2[2], -fm(w1[2], w2[1])), dy = __fmaf_rn(w1[2], w2[0], -fm(w1[0], w2[2])),
                dz = __fmaf_rn(w1[0], w2[1], -fm(w1[1], w2[0]));
    const float f = __fdiv_rn(__fsqrt_rn(fa(fa(sqf(dx), sqf(dy)), sqf(dz))), P.dis);
    const float g = __fmaf_rn(w1[2], P.axis[2], __fmaf_rn(w1[0], P.axis[0], fm(w1[1], P.axis[1])));
    const float fld1 = fmaxf(fs(g, tda), -fa(g, tda));
    const float fld2 = P.flag ? fmaxf(fs(f, fa(r, td)), -fs(f, fs(r, td))) : fs(f, r);
    return fmaxf(fld1, fld2);
  } else {
    const float x = __fmaf_rn(tx, sp[0], -P.c[0]), y = __fmaf_rn(ty, sp[1], -P.c[1]),
                z = __fmaf_rn(tz, sp[2], -P.c[2]);
    float a, b, cc;
    rotate_ref(P, x, y, z, a, b, cc);
    if constexpr (K == 2) {  // implicit_cuboid_kernel :375-421
      return fmaxf(fmaxf(fs(fabsf(a), fm(P.p[0], 0.5f)), fs(fabsf(b), fm(P.p[1], 0.5f))),
                   fs(fabsf(cc), fm(P.p[2], 0.5f)));
    } else if constexpr (K == 3) {  // implicit_cuboid_shell_kernel :435-487
      const float wx = fm(P.p[0], 0.5f), wy = fm(P.p[1], 0.5f), wz = fm(P.p[2], 0.5f), th = P.p[3];
      const float f11 = fs(fabsf(a), wx), f12 = fs(fabsf(a), fs(wx, th));
      const float f21 = fs(fabsf(b), wy), f22 = fs(fabsf(b), fs(wy, th));
      return fmaxf(fmaxf(fmaxf(f11, f21), -fmaxf(f12, f22)), fs(fabsf(cc), wz));
    } else if constexpr (K == 4) {  // implicit_torus_kernel :569-616
      const float side = fs(P.p[0], __fsqrt_rn(fa(sqf(a), sqf(b))));
      return fa(fs(sqf(cc), sqf(P.p[1])), sqf(side));
    } else if constexpr (K == 5) {  // implicit_cone_kernel :631-683
      const float br = P.p[0], hgt = P.p[1];
      const float k2 = sqf(__fdiv_rn(hgt, br));
      const float f1 = __fmaf_rn(fa(sqf(a), sqf(cc)), k2, -sqf(fs(b, hgt)));
      return fmaxf(f1, cone_slab(b, hgt));
    } else if constexpr (K == 6) {  // implicit_cone_frustum_kernel :698-750
      const float tr = P.p[0], brr = P.p[1], hgt = P.p[2];
      const float rr = __fmaf_rn(__fdiv_rn(fs(hgt, b), hgt), fs(brr, tr), tr);
      const float f1 = (float)__dsub_rn((double)fa(sqf(a), sqf(cc)), __dmul_rn((double)rr, (double)rr));
      return fmaxf(f1, cone_slab(b, hgt));
    } else {  // implicit_pyramid_frustum_kernel :501-557
      const float xwb = fm(P.p[0], 0.5f), xwt = fm(P.p[1], 0.5f), yh = P.p[2];
      const float zwb = fm(P.p[3], 0.5f), zwt = fm(P.p[4], 0.5f);
      const float ratio = __fdiv_rn(fs(yh, b), yh);
      const float hy = fm(yh, 0.5f);
      const float f1 = fs(fabsf(a), __fmaf_rn(ratio, fs(xwb, xwt), xwt));
      const float f2 = fs(fabsf(fs(b, hy)), hy);
      const float f3 = fs(fabsf(cc), __fmaf_rn(ratio, fs(zwb, zwt), zwt));
      return fmaxf(fmaxf(f1, f2), f3);
    }
  }
}

// The same fields bit for bit as the reference's kernels: written in their
// expression shapes with plain float operators, CUDA powf / sqrtf / division
// and default contraction, so that nvcc forms the same roundings and fused
// multiply-adds as in the reference's own build.  The cone kinds evaluate the
// basis per sample from the angles, as the reference does (their expressions
// around powf round differently when the basis comes from memory), one sample
// at a time (see csg_eval8).
__device__ __forceinline__ void rotate_inline(const PrimPre& P, float x, float y, float z, float& a, float& b,
                                              float& cc) {
  const float ax = P.ang[0], ay = P.ang[1], az = P.ang[2];
  const float px[3] = {(cosf(az) * cosf(ay)), (cosf(az) * sinf(ay) * sinf(ax)) - (sinf(az) * cosf(ax)),
                       (cosf(az) * sinf(ay) * cosf(ax)) + (sinf(az) * sinf(ax))};
  const float py[3] = {((sinf(az)) * cosf(ay)), (sinf(az) * sinf(ay) * sinf(ax)) + (cosf(az) * cosf(ax)),
                       (sinf(az) * sinf(ay) * cosf(ax)) - (cosf(az) * sinf(ax))};
  const float pz[3] = {(-1.0f * sinf(ay)), cosf(ay) * sinf(ax), cosf(ay) * cosf(ax)};
  a = x * px[0] + y * px[1] + z * px[2];
  b = x * py[0] + y * py[1] + z * py[2];
  cc = x * pz[0] + y * pz[1] + z * pz[2];
}

template <int K>
__device__ __forceinline__ float prim_eval_exact(const PrimPre& P, float tx, float ty, float tz, const float sp[3]) {
  if constexpr (K == 0) {
    const float x = tx * sp[0] - P.c[0], y = ty * sp[1] - P.c[1], z = tz * sp[2] - P.c[2];
    const float r = P.p[0], td = P.p[1] / 2.0;
    if (P.flag) {
      const float f1 = powf(x, 2) + powf(y, 2) + powf(z, 2) - powf((r - td), 2);
      const float f2 = powf(x, 2) + powf(y, 2) + powf(z, 2) - powf((r + td), 2);
      return max(f1 * -1.0, f2);
    }
    return powf(x, 2) + powf(y, 2) + powf(z, 2) - powf((r), 2);
  } else if constexpr (K == 1) {
    const float x1 = tx * sp[0], y1 = ty * sp[1], z1 = tz * sp[2];
    const float r = P.p[0], td = P.p[1] / 2.0, tda = P.p[2] / 2.0;
    const float w1[3] = {x1 - P.c[0], y1 - P.c[1], z1 - P.c[2]};
    const float w2[3] = {x1 - P.end[0], y1 - P.end[1], z1 - P.end[2]};
    const float d[3] = {w1[1] * w2[2] - w1[2] * w2[1], w1[2] * w2[0] - w1[0] * w2[2], w1[0] * w2[1] - w1[1] * w2[0]};
    const float e = sqrtf(powf(d[0], 2) + powf(d[1], 2) + powf(d[2], 2));
    const float f = e / P.dis;
    const float g = ((x1 - P.c[0]) * P.axis[0] + (y1 - P.c[1]) * P.axis[1] + (z1 - P.c[2]) * P.axis[2]);
    const float fld1 = max(g - tda, (g + tda) * -1);
    const float fld2 = P.flag ? (float)max((f - (r + td)), (f - (r - td)) * -1.0) : (f - (r));
    return max(fld1, fld2);
  } else {
    const float x = tx * sp[0] - P.c[0], y = ty * sp[1] - P.c[1], z = tz * sp[2] - P.c[2];
    float a, b, cc;
    if constexpr (K == 5 || K == 6) {
      rotate_inline(P, x, y, z, a, b, cc);
    } else {
      a = x * P.R[0] + y * P.R[1] + z * P.R[2];
      b = x * P.R[3] + y * P.R[4] + z * P.R[5];
      cc = __fmaf_rn(z, P.R[8], __fmaf_rn(y, P.R[7], -__fmul_rn(x, P.sy)));
    }
    if constexpr (K == 2) {
      const float xw = P.p[0] / 2.0, yw = P.p[1] / 2.0, zw = P.p[2] / 2.0;
      return max(max(fabs(a) - xw, fabs(b) - yw), fabs(cc) - zw);
    } else if constexpr (K == 3) {
      const float xw = P.p[0] / 2.0, yw = P.p[1] / 2.0, zw = P.p[2] / 2.0, th = P.p[3];
      const float f11 = fabs(a) - xw, f12 = fabs(a) - (xw - th);
      const float f21 = fabs(b) - yw, f22 = fabs(b) - (yw - th);
      const float f3 = fabs(cc) - zw;
      return max(max(max(f11, f21), (max(f12, f22)) * -1.0), f3);
    } else if constexpr (K == 4) {
      const float side = (P.p[0] - sqrtf(powf(a, 2) + powf(b, 2)));
      return powf(cc, 2) - powf(P.p[1], 2) + powf(side, 2);
    } else if constexpr (K == 5) {
      const float br = P.p[0], h = P.p[1];
      const float k2 = powf((h / br), 2);
      const float g = (b - (h / 2.0));
      const float hh = max((g - (h / 2.0)) * 100, (g + (h / 2.0)) * 100 * -1.0);
      const float f1 = ((powf((a), 2) + powf((cc), 2)) * k2) - powf((b - h), 2);
      return max(f1, hh);
    } else if constexpr (K == 6) {
      const float tr = P.p[0], brr = P.p[1], h = P.p[2];
      const float rd = ((h - b) / h) * (brr - tr);
      const float g = (b - (h / 2.0));
      const float hh = max((g - (h / 2.0)) * 100, (g + (h / 2.0)) * 100 * -1.0);
      const float f1 = ((powf((a), 2) + powf((cc), 2))) - pow((rd + tr), 2);
      return max(f1, hh);
    } else {
      const float xwb = P.p[0] / 2.0, xwt = P.p[1] / 2.0, yh = P.p[2], zwb = P.p[3] / 2.0, zwt = P.p[4] / 2.0;
      const float ratio = ((yh - b) / yh);
      const float xw = (ratio * (xwb - xwt)) + xwt;
      const float f1 = fabs(a) - xw;
      const float f2 = fabs(b - (yh / 2)) - ((yh) / 2);
      const float zw = (ratio * (zwb - zwt)) + zwt;
      const float f3 = fabs(cc) - zw;
      return max(max(f1, f2), f3);
    }
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// Per-tile primitive culling.  The scene is evaluated in tiles of 32 x 8 x 4
// samples.  For each tile every primitive gets an enclosure [L, U] of the
// values the evaluation above produces at the tile's samples: each step of the
// evaluation is a correctly rounded IEEE operation that is monotone in each
// argument (products of two varying terms are taken at the interval corners),
// so repeating the same operations on interval end points encloses the float
// results themselves, not just the real-valued function.  A small slack
// (2^-20 of the magnitudes involved, plus 1e-30) covers double-rounding
// differences in the two double-precision cone expressions and flush-to-zero.
//
// A run of consecutive operations of one kind folds a multiset with min (or
// max).  Within a union run with running upper bound M = min(hi(f), U_k), a
// primitive with L_k > M is strictly above the run's result at every sample
// of the tile, so dropping it changes no result bit (the minimum of the rest
// is the same value; it is never a zero that could tie with another).  The
// same holds mirrored for subtract (-g_k) and intersect runs.  The kept
// primitives are evaluated in their original order.
// ---------------------------------------------------------------------------
namespace {

struct Iv {
  float lo, hi;
};

__device__ __forceinline__ Iv iv_abs(Iv a) {
  if (a.lo >= 0.0f) return a;
  if (a.hi <= 0.0f) return {-a.hi, -a.lo};
  return {0.0f, fmaxf(-a.lo, a.hi)};
}
__device__ __forceinline__ Iv iv_sq(Iv a) {
  const Iv m = iv_abs(a);
  return {fm(m.lo, m.lo), fm(m.hi, m.hi)};
}
__device__ __forceinline__ Iv iv_mul_c(Iv a, float c) {
  const float u = fm(a.lo, c), v = fm(a.hi, c);
  return {fminf(u, v), fmaxf(u, v)};
}
__device__ __forceinline__ Iv iv_mul(Iv a, Iv b) {
  const float p0 = fm(a.lo, b.lo), p1 = fm(a.lo, b.hi), p2 = fm(a.hi, b.lo), p3 = fm(a.hi, b.hi);
  return {fminf(fminf(p0, p1), fminf(p2, p3)), fmaxf(fmaxf(p0, p1), fmaxf(p2, p3))};
}
__device__ __forceinline__ Iv iv_add3(Iv a, Iv b, Iv c) { return {fa(fa(a.lo, b.lo), c.lo), fa(fa(a.hi, b.hi), c.hi)}; }
__device__ __forceinline__ Iv iv_sub(Iv a, Iv b) { return {fs(a.lo, b.hi), fs(a.hi, b.lo)}; }
__device__ __forceinline__ Iv iv_subc(Iv a, float c) { return {fs(a.lo, c), fs(a.hi, c)}; }
__device__ __forceinline__ Iv iv_neg(Iv a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ Iv iv_max(Iv a, Iv b) { return {fmaxf(a.lo, b.lo), fmaxf(a.hi, b.hi)}; }
__device__ __forceinline__ float iv_mag(Iv a) { return fa(fabsf(a.lo), fabsf(a.hi)); }
// Rotated coordinate: fa(fa(fm(x, r0), fm(y, r1)), fm(z, r2)).
__device__ __forceinline__ Iv iv_row(const Iv w[3], const float* r) {
  return iv_add3(iv_mul_c(w[0], r[0]), iv_mul_c(w[1], r[1]), iv_mul_c(w[2], r[2]));
}
// h of the cone kernels, in double as there: with g = (float)(b - hgt/2),
// h = max((g - hgt/2) * 100, -(g + hgt/2) * 100).  The first piece increases
// with b and the second decreases, so h over [b.lo, b.hi] lies between the
// maxima of the pieces taken at opposite ends.
__device__ __forceinline__ Iv cone_h_iv(Iv b, float hgt, float& mag) {
  const float gl = (float)((double)b.lo - (double)hgt / 2.0), gh = (float)((double)b.hi - (double)hgt / 2.0);
  const float p1l = (float)(((double)gl - (double)hgt / 2.0) * 100.0);
  const float p1h = (float)(((double)gh - (double)hgt / 2.0) * 100.0);
  const float p2l = (float)(((double)gh + (double)hgt / 2.0) * 100.0 * -1.0);
  const float p2h = (float)(((double)gl + (double)hgt / 2.0) * 100.0 * -1.0);
  mag = fa(mag, fa(fa(fabsf(p1l), fabsf(p1h)), fa(fabsf(p2l), fabsf(p2h))));
  return {fmaxf(p1l, p2l), fmaxf(p1h, p2h)};
}

// Enclosure of prim_eval_k over the box [blo, bhi] of sample positions, or
// (-inf, +inf) when any step is not finite.
__device__ float2 prim_bounds(const PrimPre& P, const float* blo, const float* bhi) {
  Iv w[3];
  for (int a = 0; a < 3; ++a) w[a] = {fs(blo[a], P.c[a]), fs(bhi[a], P.c[a])};
  float mag = fa(fa(iv_mag(w[0]), iv_mag(w[1])), iv_mag(w[2]));
  Iv g;
  switch (P.kind) {
    case 0: {
      const Iv x2 = iv_sq(w[0]), y2 = iv_sq(w[1]), z2 = iv_sq(w[2]);
      const Iv d2 = iv_add3(x2, y2, z2);
      const float r = P.p[0], t = P.p[1] * 0.5f;
      if (P.flag) {
        const float A = sqf(fs(r, t)), B = sqf(fa(r, t));
        g = iv_max(iv_neg(iv_subc(d2, A)), iv_subc(d2, B));
        mag = fa(mag, fa(A, B));
      } else {
        g = iv_subc(d2, sqf(r));
        mag = fa(mag, sqf(r));
      }
      mag = fa(mag, d2.hi);
      break;
    }
    case 1: {
      const float r = P.p[0], td = P.p[1] * 0.5f, tda = P.p[2] * 0.5f;
      Iv v[3];
      for (int a = 0; a < 3; ++a) v[a] = {fs(blo[a], P.end[a]), fs(bhi[a], P.end[a])};
      const Iv dx = iv_sub(iv_mul(w[1], v[2]), iv_mul(w[2], v[1]));
      const Iv dy = iv_sub(iv_mul(w[2], v[0]), iv_mul(w[0], v[2]));
      const Iv dz = iv_sub(iv_mul(w[0], v[1]), iv_mul(w[1], v[0]));
      const Iv s2 = iv_add3(iv_sq(dx), iv_sq(dy), iv_sq(dz));
      const Iv e = {__fsqrt_rn(s2.lo), __fsqrt_rn(s2.hi)};
      const Iv f = {__fdiv_rn(e.lo, P.dis), __fdiv_rn(e.hi, P.dis)};
      const Iv ga = iv_row(w, P.axis);
      const Iv fld1 = iv_max(iv_subc(ga, tda), iv_neg({fa(ga.lo, tda), fa(ga.hi, tda)}));
      Iv fld2;
      if (P.flag) fld2 = iv_max(iv_subc(f, fa(r, td)), iv_neg(iv_subc(f, fs(r, td))));
      else fld2 = iv_subc(f, r);
      g = iv_max(fld1, fld2);
      mag = fa(fa(fa(mag, s2.hi), iv_mag(f)), fa(fa(iv_mag(ga), fabsf(r)), fa(fabsf(td), fabsf(tda))));
      mag = fa(mag, fa(fa(iv_mag(v[0]), iv_mag(v[1])), iv_mag(v[2])));
      break;
    }
    default: {
      const Iv a = iv_row(w, P.R), b = iv_row(w, P.R + 3), cc = iv_row(w, P.R + 6);
      mag = fa(mag, fa(fa(iv_mag(a), iv_mag(b)), iv_mag(cc)));
      const Iv aa = iv_abs(a), ab = iv_abs(b), ac = iv_abs(cc);
      switch (P.kind) {
        case 2:
          g = iv_max(iv_max(iv_subc(aa, P.p[0] * 0.5f), iv_subc(ab, P.p[1] * 0.5f)), iv_subc(ac, P.p[2] * 0.5f));
          break;
        case 3: {
          const float wx = P.p[0] * 0.5f, wy = P.p[1] * 0.5f, wz = P.p[2] * 0.5f, th = P.p[3];
          const Iv f11 = iv_subc(aa, wx), f12 = iv_subc(aa, fs(wx, th));
          const Iv f21 = iv_subc(ab, wy), f22 = iv_subc(ab, fs(wy, th));
          g = iv_max(iv_max(iv_max(f11, f21), iv_neg(iv_max(f12, f22))), iv_subc(ac, wz));
          mag = fa(mag, fa(fa(fabsf(wx), fabsf(wy)), fa(fabsf(wz), fabsf(th))));
          break;
        }
        case 4: {
          const Iv s2 = {fa(sqf(aa.lo), sqf(ab.lo)), fa(sqf(aa.hi), sqf(ab.hi))};
          const Iv side = {fs(P.p[0], __fsqrt_rn(s2.hi)), fs(P.p[0], __fsqrt_rn(s2.lo))};
          const Iv q = iv_sq(side);
          g = {fa(fs(sqf(ac.lo), sqf(P.p[1])), q.lo), fa(fs(sqf(ac.hi), sqf(P.p[1])), q.hi)};
          mag = fa(fa(mag, s2.hi), fa(fa(q.hi, sqf(ac.hi)), sqf(P.p[1])));
          break;
        }
        case 5: {
          const float br = P.p[0], hgt = P.p[1];
          const float k2 = sqf(__fdiv_rn(hgt, br));
          const Iv q = {fm(fa(sqf(aa.lo), sqf(ac.lo)), k2), fm(fa(sqf(aa.hi), sqf(ac.hi)), k2)};
          const Iv d = iv_sq(iv_subc(b, hgt));
          const Iv f1 = {fs(q.lo, d.hi), fs(q.hi, d.lo)};
          const Iv hh = cone_h_iv(b, hgt, mag);
          g = iv_max(f1, hh);
          mag = fa(mag, fa(fa(q.hi, d.hi), fabsf(k2)));
          break;
        }
        case 6: {
          const float tr = P.p[0], brr = P.p[1], hgt = P.p[2];
          const float u1 = fm(__fdiv_rn(fs(hgt, b.lo), hgt), fs(brr, tr));
          const float u2 = fm(__fdiv_rn(fs(hgt, b.hi), hgt), fs(brr, tr));
          const Iv rd = {fminf(u1, u2), fmaxf(u1, u2)};
          const Iv rrf = {fa(rd.lo, tr), fa(rd.hi, tr)};
          const Iv m = iv_abs(rrf);
          const Iv A = {fa(sqf(aa.lo), sqf(ac.lo)), fa(sqf(aa.hi), sqf(ac.hi))};
          const Iv f1 = {(float)((double)A.lo - (double)m.hi * (double)m.hi),
                         (float)((double)A.hi - (double)m.lo * (double)m.lo)};
          g = iv_max(f1, cone_h_iv(b, hgt, mag));
          mag = fa(mag, fa(A.hi, sqf(m.hi)));
          break;
        }
        default: {
          const float xwb = P.p[0] * 0.5f, xwt = P.p[1] * 0.5f, yh = P.p[2];
          const float zwb = P.p[3] * 0.5f, zwt = P.p[4] * 0.5f;
          const float r1 = __fdiv_rn(fs(yh, b.lo), yh), r2 = __fdiv_rn(fs(yh, b.hi), yh);
          const Iv ratio = {fminf(r1, r2), fmaxf(r1, r2)};
          const Iv xw0 = iv_mul_c(ratio, fs(xwb, xwt)), zw0 = iv_mul_c(ratio, fs(zwb, zwt));
          const Iv xw = {fa(xw0.lo, xwt), fa(xw0.hi, xwt)}, zw = {fa(zw0.lo, zwt), fa(zw0.hi, zwt)};
          const float hy = __fdiv_rn(yh, 2.0f);
          const Iv f1 = iv_sub(aa, xw);
          const Iv f2 = iv_subc(iv_abs(iv_subc(b, hy)), hy);
          const Iv f3 = iv_sub(ac, zw);
          g = iv_max(iv_max(f1, f2), f3);
          mag = fa(fa(mag, fa(iv_mag(ratio), iv_mag(xw))), fa(fa(iv_mag(zw), fabsf(hy)), fa(fabsf(xwb), fabsf(zwb))));
          break;
        }
      }
    }
  }
  mag = fa(mag, iv_mag(g));
  const float slack = fa(fm(mag, 0x1p-20f), 1e-30f);
  if (!(fabsf(slack) <= FLT_MAX)) return make_float2(-INFINITY, INFINITY);
  return make_float2(fs(g.lo, slack), fa(g.hi, slack));
}

__device__ __forceinline__ uint32_t csg_op(uint32_t op) { return op == 1 ? 1u : (op == 2 ? 2u : 0u); }

__device__ __forceinline__ float warp_min(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// One warp picks, in order, the primitives that can change the samples of its
// tile, from their enclosures lu[] (x = L, y = U).  run_end[i] is the end of
// the run of equal operations starting at i.  Returns the count; the indices
// go to list[].
// flo_out, fhi_out: an enclosure of the folded field over the tile.
__device__ uint32_t csg_cull_warp(const PrimPre* pre, const uint16_t* run_end, const float2* lu, uint32_t n,
                                  uint8_t* list, uint32_t lane, float& flo_out, float& fhi_out) {
  float flo = INFINITY, fhi = INFINITY;  // the running field starts at +inf
  uint32_t cnt = 0;
  const uint32_t below = (1u << lane) - 1u;
  for (uint32_t i = 0; i < n;) {
    const uint32_t j = run_end[i], op = csg_op(pre[i].op);
    // union: items g_k, threshold M = min(hi f, U_k), drop L_k > M
    // subtract: items -g_k in [-U_k, -L_k], threshold m = max(lo f, -U_k), drop -L_k < m
    // intersect: items g_k, threshold m = max(lo f, L_k), drop U_k < m
    float t = op == 0 ? fhi : flo;
    for (uint32_t k = i + lane; k < j; k += 32) {
      const float2 b = lu[k];
      t = op == 0 ? fminf(t, b.y) : (op == 1 ? fmaxf(t, -b.y) : fmaxf(t, b.x));
    }
    t = op == 0 ? warp_min(t) : warp_max(t);
    float e = op == 0 ? INFINITY : -INFINITY;  // new lower (union) or upper bound of the kept items
    for (uint32_t base = i; base < j; base += 32) {
      const uint32_t k = base + lane;
      bool keep = false;
      if (k < j) {
        const float2 b = lu[k];
        if (op == 0) {
          keep = !(b.x > t);
          if (keep) e = fminf(e, b.x);
        } else if (op == 1) {
          keep = !(-b.x < t);
          if (keep) e = fmaxf(e, -b.x);
        } else {
          keep = !(b.y < t);
          if (keep) e = fmaxf(e, b.y);
        }
      }
      const uint32_t m = __ballot_sync(0xffffffffu, keep);
      if (keep) list[cnt + __popc(m & below)] = (uint8_t)k;
      cnt += __popc(m);
    }
    if (op == 0) {
      flo = fminf(flo, warp_min(e));
      fhi = t;
    } else {
      fhi = fmaxf(fhi, warp_max(e));
      flo = t;
    }
    i = j;
  }
  __syncwarp();
  flo_out = flo;
  fhi_out = fhi;
  return cnt;
}

// A warp's tile: 32 samples along x (one per lane) by 8 rows (y) by 8 planes (z).
constexpr uint32_t kCsgTx = GCM_CSG_TILE_X, kCsgTy = GCM_CSG_TILE_Y, kCsgTz = GCM_CSG_TILE_Z, kCsgWarps = 8;

__device__ __forceinline__ float csg_coord(uint32_t i, float o, float s) { return fm(fs((float)i, o), s); }

__device__ __forceinline__ float csg_fold(uint32_t op, float f, float g) {
  return op == 1 ? fmaxf(f, -g) : (op == 2 ? fmaxf(f, g) : fminf(f, g));
}

template <int K, bool EXACT>
__device__ __forceinline__ void csg_eval8(const PrimPre& P, uint32_t op, float tX, float tY,
                                          const float (&tZ)[kCsgTz], const float sp[3], float (&f)[kCsgTz]) {
  if constexpr (!EXACT) {
#pragma unroll
    for (uint32_t q = 0; q < kCsgTz; ++q) f[q] = csg_fold(op, f[q], prim_eval_k<K>(P, tX, tY, tZ[q], sp));
  } else if constexpr (K == 5 || K == 6) {
    // one sample per iteration: unrolled, the samples' shared terms change
    // how nvcc contracts these expressions
#pragma unroll 1
    for (uint32_t q = 0; q < kCsgTz; ++q) f[q] = csg_fold(op, f[q], prim_eval_exact<K>(P, tX, tY, tZ[q], sp));
  } else {
#pragma unroll
    for (uint32_t q = 0; q < kCsgTz; ++q) f[q] = csg_fold(op, f[q], prim_eval_exact<K>(P, tX, tY, tZ[q], sp));
  }
}

}  // namespace

template <bool EXACT>
__global__ void __launch_bounds__(kCsgWarps * 32, 4) csg_kernel(CsgParams p) {
  extern __shared__ __align__(16) unsigned char csg_smem[];
  const uint32_t n = p.n;  // at most 256 (checked by the caller)
  PrimPre* s_pre = reinterpret_cast<PrimPre*>(csg_smem);
  float2* s_lu = reinterpret_cast<float2*>(csg_smem + (size_t)n * sizeof(PrimPre));
  uint16_t* s_run = reinterpret_cast<uint16_t*>(s_lu + (size_t)kCsgWarps * n);
  uint8_t* s_perm = reinterpret_cast<uint8_t*>(s_run + n);
  uint8_t* s_list = s_perm + n;
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  for (uint32_t i = tid; i < n; i += blockDim.x) prim_setup<EXACT>(p.prims[i], s_pre[i]);
  __syncthreads();
  for (uint32_t i = tid; i < n; i += blockDim.x) {
    const uint32_t op = csg_op(s_pre[i].op), kind = min(s_pre[i].kind, 7u);
    // end of the run of equal operations that starts here (read only at run starts)
    uint32_t j = i + 1;
    while (j < n && csg_op(s_pre[j].op) == op) ++j;
    s_run[i] = (uint16_t)j;
    // place in kind order, so that a warp's lanes mostly share a kind when
    // they compute enclosures
    uint32_t rank = 0;
    for (uint32_t k = 0; k < n; ++k) {
      const uint32_t kk = min(s_pre[k].kind, 7u);
      rank += (kk < kind || (kk == kind && k < i)) ? 1u : 0u;
    }
    s_perm[rank] = (uint8_t)i;
  }
  __syncthreads();
  float2* lu = s_lu + (size_t)warp * n;
  uint8_t* list = s_list + (size_t)warp * n;
  const uint32_t tx = (p.nx + kCsgTx - 1) / kCsgTx, ty = (p.ny + kCsgTy - 1) / kCsgTy;
  const uint32_t tz = (p.nz + kCsgTz - 1) / kCsgTz;
  const uint64_t tiles = (uint64_t)tx * ty * tz;
  const uint64_t stride = (uint64_t)gridDim.x * kCsgWarps;
  for (uint64_t t = (uint64_t)blockIdx.x * kCsgWarps + warp; t < tiles; t += stride) {
    const uint32_t bx = (uint32_t)(t % tx), by = (uint32_t)((t / tx) % ty), bz = (uint32_t)(t / ((uint64_t)tx * ty));
    const uint32_t x0 = bx * kCsgTx, y0 = by * kCsgTy, z0 = bz * kCsgTz;
    {
      const uint32_t i0[3] = {x0, y0, z0};
      const uint32_t i1[3] = {min(x0 + kCsgTx - 1, p.nx - 1), min(y0 + kCsgTy - 1, p.ny - 1),
                              min(z0 + kCsgTz - 1, p.nz - 1)};
      float blo[3], bhi[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        // sample positions are monotone in the index
        const float u = csg_coord(i0[a], p.origin[a], p.spacing[a]), v = csg_coord(i1[a], p.origin[a], p.spacing[a]);
        blo[a] = fminf(u, v);
        bhi[a] = fmaxf(u, v);
        if (!(fabsf(u) <= FLT_MAX && fabsf(v) <= FLT_MAX)) {
          blo[a] = -INFINITY;
          bhi[a] = INFINITY;
        }
      }
      for (uint32_t c = lane; c < n; c += 32) {
        const uint32_t k = s_perm[c];
        lu[k] = prim_bounds(s_pre[k], blo, bhi);
      }
    }
    __syncwarp();
    float flo, fhi;
    const uint32_t cnt = csg_cull_warp(s_pre, s_run, lu, n, list, lane, flo, fhi);
    // every sample of the tile lies in [flo, fhi] (NaN bounds compare false: mixed)
    if (p.tile_state && lane == 0)
      p.tile_state[t] = fhi < p.iso ? kTileInside : (flo >= p.iso ? kTileOutside : kTileMixed);
    const uint32_t px = x0 + lane;
    // sample offsets index - origin; the primitives form their positions
    const float tX = fs((float)px, p.origin[0]);
    float tZ[kCsgTz];
#pragma unroll
    for (uint32_t q = 0; q < kCsgTz; ++q) tZ[q] = fs((float)(z0 + q), p.origin[2]);
#pragma unroll 1
    for (uint32_t r = 0; r < kCsgTy; ++r) {
      const uint32_t py = y0 + r;
      if (py >= p.ny) break;  // warp-uniform
      const float tY = fs((float)py, p.origin[1]);
      float f[kCsgTz];
#pragma unroll
      for (uint32_t q = 0; q < kCsgTz; ++q) f[q] = INFINITY;
      for (uint32_t j = 0; j < cnt; ++j) {
        const PrimPre& P = s_pre[list[j]];
        const uint32_t op = P.op;
        switch (P.kind) {
          case 0: csg_eval8<0, EXACT>(P, op, tX, tY, tZ, p.spacing, f); break;
          case 1: csg_eval8<1, EXACT>(P, op, tX, tY, tZ, p.spacing, f); break;
          case 2: csg_eval8<2, EXACT>(P, op, tX, tY, tZ, p.spacing, f); break;
          case 3: csg_eval8<3, EXACT>(P, op, tX, tY, tZ, p.spacing, f); break;
          case 4: csg_eval8<4, EXACT>(P, op, tX, tY, tZ, p.spacing, f); break;
          case 5: csg_eval8<5, EXACT>(P, op, tX, tY, tZ, p.spacing, f); break;
          case 6: csg_eval8<6, EXACT>(P, op, tX, tY, tZ, p.spacing, f); break;
          default: csg_eval8<7, EXACT>(P, op, tX, tY, tZ, p.spacing, f); break;
        }
      }
      if (px < p.nx) {
        float* out = p.out + ((uint64_t)z0 * p.ny + py) * p.nx + px;
        const uint64_t plane = (uint64_t)p.ny * p.nx;
#pragma unroll
        for (uint32_t q = 0; q < kCsgTz; ++q)
          if (z0 + q < p.nz) out[q * plane] = f[q];
      }
    }
    __syncwarp();  // lu[] and list[] are rewritten for the next tile
  }
}

// ---------------------------------------------------------------------------
// Band normalisation (GPU_buffer_normalise_four, src/lattice_files/Gratings.cu:
// 1579-1617).  Floats are mapped to order-preserving unsigned keys for the
// atomic min/max; both start from the key of 0.0 (the reference's reduction
// starts from {0,0}, Min_reduction_lattice :1439-1495).
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned int f2key(float f) {
  const unsigned int u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float key2f(unsigned int k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

__global__ void minmax_init_kernel(unsigned int* enc) {
  enc[0] = f2key(0.0f);
  enc[1] = f2key(0.0f);
}

__global__ void __launch_bounds__(256) minmax_kernel(const float* f, uint64_t n, unsigned int* enc_min,
                                                     unsigned int* enc_max) {
  unsigned int lo = f2key(0.0f), hi = f2key(0.0f);
  const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x, stride = (uint64_t)gridDim.x * blockDim.x;
  uint64_t head = 0;  // samples before the first 16-byte boundary
  if (((uintptr_t)f & 15u) == 0) {
    // 16-byte loads: four samples per load
    const float4* f4 = reinterpret_cast<const float4*>(f);
    const uint64_t n4 = n / 4;
    for (uint64_t i = tid; i < n4; i += stride) {
      const float4 v = __ldg(f4 + i);
      const unsigned int k0 = f2key(v.x), k1 = f2key(v.y), k2 = f2key(v.z), k3 = f2key(v.w);
      lo = min(min(lo, min(k0, k1)), min(k2, k3));
      hi = max(max(hi, max(k0, k1)), max(k2, k3));
    }
    head = 4 * n4;
  }
  for (uint64_t i = head + tid; i < n; i += stride) {
    const unsigned int k = f2key(__ldg(f + i));
    lo = min(lo, k);
    hi = max(hi, k);
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if ((threadIdx.x & 31u) == 0) {
    atomicMin(enc_min, lo);
    atomicMax(enc_max, hi);
  }
}

// One warp per sample row: the row's (y, z) and boundary test once, then x,
// four samples per 16-byte access where the rows allow it.
__device__ __forceinline__ void band_sample(float v, float a, float b, float lo, float hi, bool edge, float& m,
                                            float& k) {
  k = __fdiv_rn(fs(v, a), fs(b, a));
  if (edge) {
    m = 0.0f;
    k = 0.0f;
  } else {
    m = (k >= lo && k <= hi) ? 1.0f : 0.0f;
  }
}

__global__ void __launch_bounds__(256) band_map_kernel(const float* f, uint32_t nx, uint32_t ny, uint32_t nz,
                                                       const unsigned int* enc, float lo, float hi, float* label,
                                                       float* norm_field) {
  const float a = key2f(enc[0]), b = key2f(enc[1]);
  const uint32_t rows = ny * nz, lane = threadIdx.x & 31u;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  const bool vec = (nx & 3u) == 0 && ((((uintptr_t)f) | ((uintptr_t)label) | ((uintptr_t)norm_field)) & 15u) == 0;
  for (uint32_t row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); row < rows; row += warps) {
    const uint32_t y = row % ny, z = row / ny;
    const bool edge_row = y == 0 || y == ny - 1 || z == 0 || z == nz - 1;
    const uint64_t base = (uint64_t)row * nx;
    if (vec) {
      const float4* f4 = reinterpret_cast<const float4*>(f + base);
      float4* l4 = reinterpret_cast<float4*>(label + base);
      float4* k4 = reinterpret_cast<float4*>(norm_field + base);
      for (uint32_t x4 = lane; x4 < nx / 4; x4 += 32) {
        const float4 v = __ldg(f4 + x4);
        const uint32_t x = 4 * x4;
        float4 m, k;
        band_sample(v.x, a, b, lo, hi, edge_row || x == 0, m.x, k.x);
        band_sample(v.y, a, b, lo, hi, edge_row, m.y, k.y);
        band_sample(v.z, a, b, lo, hi, edge_row, m.z, k.z);
        band_sample(v.w, a, b, lo, hi, edge_row || x + 3 == nx - 1, m.w, k.w);
        l4[x4] = m;
        k4[x4] = k;
      }
    } else {
      for (uint32_t x = lane; x < nx; x += 32) {
        float m, k;
        band_sample(__ldg(f + base + x), a, b, lo, hi, edge_row || x == 0 || x == nx - 1, m, k);
        label[base + x] = m;
        norm_field[base + x] = k;
      }
    }
  }
}

// device_bufferthree (src/lattice_files/Gratings.cu:1071-1087): v -> a1 + b1 *
// (v - min) / (max - min), with the min/max keys of minmax_kernel (whose
// reduction starts from 0, like GPU_buffer_normalise_three's, :1539-1572); the
// reference build fuses a1 + b1 * k.  Four samples per thread where the
// buffers allow 16-byte accesses.
__device__ __forceinline__ float range_map(float v, float a, float b, float a1, float b1) {
  return __fmaf_rn(b1, __fdiv_rn(fs(v, a), fs(b, a)), a1);
}

__global__ void __launch_bounds__(256) range_map_kernel(const float* in, float* out, uint64_t n,
                                                        const unsigned int* enc, float a1, float b1) {
  const float a = key2f(enc[0]), b = key2f(enc[1]);
  const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x, stride = (uint64_t)gridDim.x * blockDim.x;
  if ((((uintptr_t)in | (uintptr_t)out) & 15u) == 0) {
    const uint64_t n4 = n / 4;
    for (uint64_t i = tid; i < n4; i += stride) {
      float4 v = reinterpret_cast<const float4*>(in)[i];
      v.x = range_map(v.x, a, b, a1, b1);
      v.y = range_map(v.y, a, b, a1, b1);
      v.z = range_map(v.z, a, b, a1, b1);
      v.w = range_map(v.w, a, b, a1, b1);
      reinterpret_cast<float4*>(out)[i] = v;
    }
    for (uint64_t i = 4 * n4 + tid; i < n; i += stride) out[i] = range_map(in[i], a, b, a1, b1);
  } else {
    for (uint64_t i = tid; i < n; i += stride) out[i] = range_map(in[i], a, b, a1, b1);
  }
}

// primitive_field_kernel (src/lattice_files/Gratings.cu:1695-1725): a lattice
// sample becomes FLT_MAX where the retained model does not hold it (fixed:
// the record's sign val > -1, i.e. outside or never touched) or, otherwise,
// where the live primitive field is >= 0 (dynamic); other samples keep their
// value.  NaN primitive values keep the sample, as in the reference.
__global__ void __launch_bounds__(256) lattice_mask_kernel(const gcm_csg_point* __restrict__ acc,
                                                           const float* __restrict__ prim, float* lat, uint64_t n,
                                                           uint32_t fixed) {
  const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x, stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = tid; i < n; i += stride) {
    const bool out = fixed ? __ldg(&acc[i].val) > -1 : __ldg(prim + i) >= 0.0f;
    if (out) lat[i] = FLT_MAX;
  }
}

// ---------------------------------------------------------------------------
// Launch wrappers.
// ---------------------------------------------------------------------------
cudaError_t launch_unit_cell(uint32_t type, uint32_t nx, uint32_t ny, uint32_t nz, float* out, uint32_t blocks,
                             cudaStream_t st) {
  // a whole number of column chunks per grid (at least one of each)
  const uint64_t W = unit_cell_width(nx), xchunks = (nx + W - 1) / W;
  const uint64_t items = xchunks * (((uint64_t)ny * nz + kUnitRows - 1) / kUnitRows);
  uint64_t g = std::min<uint64_t>(std::max<uint64_t>(blocks, xchunks), items);
  g = std::max<uint64_t>(g / xchunks, 1) * xchunks;
  unit_cell_kernel<<<(uint32_t)std::min<uint64_t>(g, 1ull << 30), 256, 0, st>>>(type, nx, ny, nz, out);
  return cudaGetLastError();
}

// Rows per warp for lattice_rows_kernel: the most of {8, 4, 2, 1} whose slices
// fit kRowSmem and that still leave 32 warps of row groups per SM; 1 when one
// row's slices fit kRowSmemWide (opt-in shared memory); 0 when not even that
// (the unstaged kernel then runs).
uint32_t lattice_rows_per_warp(uint32_t cx, uint32_t rows, uint32_t sm_count) {
  for (uint32_t R = 8; R >= 1; R /= 2) {
    if (row_smem_bytes(R, cx) > kRowSmem) continue;
    if (R == 1 || (uint64_t)(rows + R - 1) / R >= (uint64_t)sm_count * 32) return R;
  }
  if (row_smem_bytes(1, cx) <= kRowSmemWide) return 1;  // a wide control grid, opt-in shared memory
  return 0;
}

template <uint32_t R>
static cudaError_t launch_rows(const LatticeParams& p, cudaStream_t st) {
  const uint64_t groups = ((uint64_t)p.ny * p.nz + R - 1) / R;
  // at most 2^26 CTAs, so the kernel's 32-bit warp stride cannot wrap (the
  // group loop covers the rest)
  const uint32_t blocks = (uint32_t)std::min<uint64_t>((groups + kRowWarps - 1) / kRowWarps, 1u << 26);
  const size_t smem = row_smem_bytes(R, p.cx);
  if (smem > kRowSmem) {
    // every caller sets the same value (the kernel's full opt-in limit)
    int dev = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(lattice_rows_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    if (e != cudaSuccess) return e;
  }
  lattice_rows_kernel<R><<<blocks, kRowWarps * 32, smem, st>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_lattice(const LatticeParams& p, float* blend_buf, uint32_t prep_blocks, uint32_t blocks,
                           uint32_t sm_count, cudaStream_t st) {
  if (p.mode == 1) {
    lattice_prep_kernel<<<prep_blocks, 256, 0, st>>>(p, blend_buf);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    LatticeParams q = p;
    q.blend = blend_buf;
    if (p.cx <= kBlendWarpCxWide) {
      // a sample row per warp; many CTAs, so the block scheduler balances the SMs
      const uint64_t rows = (uint64_t)p.ny * p.nz;
      const uint32_t wblocks = (uint32_t)std::min<uint64_t>((rows + kBlendWarps - 1) / kBlendWarps, 1u << 26);
      const size_t smem = (size_t)kBlendWarps * 4 * p.cx * 4 * sizeof(float4);
      if (p.cx > kBlendWarpCx) {
        // every caller sets the same value (the kernel's full opt-in limit)
        int dev = 0, optin = 0;
        e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        if (e == cudaSuccess)
          e = cudaFuncSetAttribute(lattice_blend_warp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        if (e != cudaSuccess) return e;
      }
      lattice_blend_warp_kernel<<<wblocks, kBlendWarps * 32, smem, st>>>(q);
    } else {
      lattice_blend_kernel<<<blocks, 256, 0, st>>>(q);
    }
  } else {
    switch (lattice_rows_per_warp(p.cx, p.ny * p.nz, sm_count)) {
      case 8: return launch_rows<8>(p, st);
      case 4: return launch_rows<4>(p, st);
      case 2: return launch_rows<2>(p, st);
      case 1: return launch_rows<1>(p, st);
      default: lattice_params_kernel<<<blocks, 256, 0, st>>>(p);
    }
  }
  return cudaGetLastError();
}

cudaError_t launch_lattice_batch(const BatchLattice* inst, uint32_t n_inst, uint64_t total_groups, uint32_t blocks,
                                 bool any_wide, cudaStream_t st) {
  lattice_params_batch_kernel<true><<<blocks, 256, 0, st>>>(inst, n_inst, total_groups);
  if (any_wide) {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    lattice_params_batch_kernel<false><<<blocks, 256, 0, st>>>(inst, n_inst, total_groups);
  }
  return cudaGetLastError();
}

uint64_t csg_tiles(uint32_t nx, uint32_t ny, uint32_t nz) {
  const uint64_t t = (uint64_t)((nx + kCsgTx - 1) / kCsgTx) * ((ny + kCsgTy - 1) / kCsgTy) * ((nz + kCsgTz - 1) / kCsgTz);
  return (t + kCsgWarps - 1) / kCsgWarps;  // CTAs that give every warp a tile
}

template <bool EXACT>
static cudaError_t launch_csg_form(const CsgParams& p, uint32_t sm_count, cudaStream_t st) {
  const size_t smem = (size_t)p.n * (sizeof(PrimPre) + kCsgWarps * (sizeof(float2) + 1) + sizeof(uint16_t) + 1);
  cudaError_t e = cudaSuccess;
  if (smem > 48 * 1024) {
    // up to 256 primitives take 52 KB; every caller sets the same value
    int dev = 0, optin = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(csg_kernel<EXACT>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    if (e != cudaSuccess) return e;
  }
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, csg_kernel<EXACT>, kCsgWarps * 32, smem);
  if (e != cudaSuccess) return e;
  const uint64_t want = csg_tiles(p.nx, p.ny, p.nz), cap = (uint64_t)sm_count * (uint64_t)(per_sm > 0 ? per_sm : 1);
  const uint32_t blocks = (uint32_t)(want < cap ? want : cap);
  csg_kernel<EXACT><<<blocks, kCsgWarps * 32, smem, st>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_csg(const CsgParams& p, uint32_t sm_count, cudaStream_t st) {
  return p.exact ? launch_csg_form<true>(p, sm_count, st) : launch_csg_form<false>(p, sm_count, st);
}

cudaError_t launch_normalise_range(const float* in, float* out, uint64_t n, unsigned int* enc, float a1, float b1,
                                   uint32_t blocks, cudaStream_t st) {
  minmax_init_kernel<<<1, 1, 0, st>>>(enc);
  minmax_kernel<<<blocks, 256, 0, st>>>(in, n, enc, enc + 1);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  range_map_kernel<<<blocks, 256, 0, st>>>(in, out, n, enc, a1, b1);
  return cudaGetLastError();
}

cudaError_t launch_lattice_mask(const gcm_csg_point* acc, const float* prim, float* lat, uint64_t n, bool fixed,
                                uint32_t blocks, cudaStream_t st) {
  lattice_mask_kernel<<<blocks, 256, 0, st>>>(acc, prim, lat, n, fixed ? 1u : 0u);
  return cudaGetLastError();
}

cudaError_t launch_normalise(const float* f, uint32_t nx, uint32_t ny, uint32_t nz, unsigned int* enc, float lo,
                             float hi, float* label, float* norm_field, uint32_t blocks, cudaStream_t st) {
  const uint64_t n = (uint64_t)nx * ny * nz;
  minmax_init_kernel<<<1, 1, 0, st>>>(enc);
  minmax_kernel<<<blocks, 256, 0, st>>>(f, n, enc, enc + 1);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  band_map_kernel<<<blocks, 256, 0, st>>>(f, nx, ny, nz, enc, lo, hi, label, norm_field);
  return cudaGetLastError();
}

}  // namespace gcm
