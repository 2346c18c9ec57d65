// CPU oracle for the field -> mesh path.  TEST INFRASTRUCTURE ONLY (see oracle.h).
//
// Built with -ffp-contract=off so that every floating-point operation rounds
// exactly where the code says; the places where the reference's nvcc build fuses
// a multiply and an add are written as explicit std::fma, selected by the
// `arith` pattern code (the pattern the reference's compiled kernels follow is
// pinned by the fixtures in tests/golden/, produced by running those kernels).
#include "oracle.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <limits>
#include <map>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "../gpucadforam_gb300/csrc/angle_table.h"
#include "../gpucadforam_gb300/csrc/mc_tables.h"

namespace {

constexpr unsigned kNumVerts(unsigned ci) { return gcm::row_verts(gcm::kTriRows[ci]); }

struct Arith {
  bool fuse_corner, fuse_delta;
  int lerp, cross;
};

Arith decode(uint32_t a) {
  Arith r;
  r.fuse_corner = (a & 1u) != 0;
  r.fuse_delta = (a & 2u) != 0;
  r.lerp = (int)((a >> 2) & 3u);
  r.cross = (int)((a >> 4) & 3u);
  return r;
}

int set_threads(int threads) {
#ifdef _OPENMP
  int t = threads > 0 ? threads : omp_get_max_threads();
  return t;
#else
  (void)threads;
  return 1;
#endif
}

inline uint64_t pidx(uint32_t x, uint32_t y, uint32_t z, uint32_t nx, uint32_t ny) {
  return (uint64_t)x + (uint64_t)nx * ((uint64_t)y + (uint64_t)ny * z);
}

// Voxel number -> (x,y,z): calcGridPos, src/MarchingCubes_kernel.cu:121-136.
inline void voxel_pos(uint64_t v, uint32_t nx, uint32_t ny, uint32_t& x, uint32_t& y, uint32_t& z) {
  uint64_t mx = nx - 1, my = ny - 1;
  z = (uint32_t)(v / (mx * my));
  uint64_t rem = v % (mx * my);
  y = (uint32_t)(rem / mx);
  x = (uint32_t)(rem % mx);
}

inline void corners(const float* f, uint32_t x, uint32_t y, uint32_t z, uint32_t nx, uint32_t ny, float c[8]) {
  for (int k = 0; k < 8; ++k)
    c[k] = f[pidx(x + gcm::kCornerX[k], y + gcm::kCornerY[k], z + gcm::kCornerZ[k], nx, ny)];
}

// Cube index: bit k set when corner k lies below the isovalue
// (classifyVoxel_new, src/MarchingCubes_kernel.cu:3230-3238).
inline unsigned cube_index(const float c[8], float iso) {
  unsigned ci = 0;
  for (int k = 0; k < 8; ++k) ci |= (unsigned)(c[k] < iso) << k;
  return ci;
}

// One coordinate of an edge point.  The reference forms the voxel origin as
// p = (gridPos - gridcenter) * voxelSize, each corner as p + offset, and the
// point as lerp(v_a, v_b, t) = v_a + t*(v_b - v_a)
// (src/MarchingCubes_kernel.cu:3061-3075, :1619-1629; helper_math.h:1145-1148).
// d = gridPos - gridcenter along this axis; oa/ob = corner offsets (0 or 1).
inline float corner_coord(float d, float vs, float P, int off, const Arith& A) {
  if (!off) return P;
  return A.fuse_corner ? std::fma(d, vs, vs) : P + vs;
}

inline float lerp_axis(float d, float vs, int oa, int ob, float t, const Arith& A) {
  const float P = d * vs;
  const float a = corner_coord(d, vs, P, oa, A);
  const float b = corner_coord(d, vs, P, ob, A);
  float B;
  if (A.fuse_delta && oa == 0) B = std::fma(-d, vs, b);
  else if (A.fuse_delta && ob == 0) B = std::fma(d, vs, -a);
  else B = b - a;
  switch (A.lerp) {
    case 1: return std::fma(t, B, a);
    case 2: return oa == 0 ? std::fma(d, vs, t * B) : std::fma(t, B, a);
    default: return a + t * B;
  }
}

// calcNormal(v0, v1, v2) = cross(v1 - v0, v2 - v0)
// (src/MarchingCubes_kernel.cu:1631-1637, helper_math.h:1427-1430).
inline float cross_term(float a, float b, float c, float d, int form) {  // a*b - c*d
  switch (form) {
    case 1: return std::fma(a, b, -(c * d));
    case 2: return std::fma(-c, d, a * b);
    default: return a * b - c * d;
  }
}

inline void normal_of(const float* v0, const float* v1, const float* v2, int form, float n[3]) {
  float e0[3] = {v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2]};
  float e1[3] = {v2[0] - v0[0], v2[1] - v0[1], v2[2] - v0[2]};
  n[0] = cross_term(e0[1], e1[2], e0[2], e1[1], form);
  n[1] = cross_term(e0[2], e1[0], e0[0], e1[2], form);
  n[2] = cross_term(e0[0], e1[1], e0[1], e1[0], form);
}

// Plain edge point: t = (iso - f_a) / (f_b - f_a) (vertexInterp4, :1619-1629).
inline void edge_point_plain(const uint32_t g[3], const float* vs, const float* gc, int e, const float c[8], float iso,
                             const Arith& A, float out[3]) {
  const int ka = gcm::kEdgeA[e], kb = gcm::kEdgeB[e];
  const float t = (iso - c[ka]) / (c[kb] - c[ka]);
  const int oa[3] = {gcm::kCornerX[ka], gcm::kCornerY[ka], gcm::kCornerZ[ka]};
  const int ob[3] = {gcm::kCornerX[kb], gcm::kCornerY[kb], gcm::kCornerZ[kb]};
  for (int ax = 0; ax < 3; ++ax) {
    const float d = (float)g[ax] - gc[ax];
    out[ax] = lerp_axis(d, vs[ax], oa[ax], ob[ax], t, A);
  }
}

// Band edge point (vertexInterp2_new, src/MarchingCubes_kernel.cu:3593-3674): only
// edges whose endpoint labels are {0,1} are interpolated; the endpoints are ordered
// so that f0 <= f1; the point snaps to an endpoint when it is within 0.0005 of a
// band edge, and otherwise lerps at the band edge crossed.  Where the reference
// leaves t unset (no branch taken) this restatement uses t = 0.
inline void edge_point_band(const uint32_t g[3], const float* vs, const float* gc, int e, const float lab[8],
                            const float fv[8], float lo, float hi, const Arith& A, float out[3]) {
  int ka = gcm::kEdgeA[e], kb = gcm::kEdgeB[e];
  const float id0 = lab[ka], id1 = lab[kb];
  float f0 = fv[ka], f1 = fv[kb];
  const bool crossing = (id0 == 1 && id1 == 0) || (id0 == 0 && id1 == 1);
  if (crossing && f1 < f0) {
    std::swap(ka, kb);
    std::swap(f0, f1);
  }
  const int oa[3] = {gcm::kCornerX[ka], gcm::kCornerY[ka], gcm::kCornerZ[ka]};
  const int ob[3] = {gcm::kCornerX[kb], gcm::kCornerY[kb], gcm::kCornerZ[kb]};
  float pa[3], pb[3];
  for (int ax = 0; ax < 3; ++ax) {
    const float d = (float)g[ax] - gc[ax];
    const float P = d * vs[ax];
    pa[ax] = corner_coord(d, vs[ax], P, oa[ax], A);
    pb[ax] = corner_coord(d, vs[ax], P, ob[ax], A);
  }
  float t = 0.0f;  // the reference leaves t unset when no branch applies
  if (crossing) {
    for (int side = 0; side < 2; ++side) {
      const float lev = side ? hi : lo;
      if ((f1 >= lev) && (f0 <= lev)) {
        if (std::fabs(lev - f0) < 0.0005) { std::memcpy(out, pa, sizeof(pa)); return; }
        if (std::fabs(lev - f1) < 0.0005) { std::memcpy(out, pb, sizeof(pb)); return; }
        if (std::fabs(f1 - f0) < 0.0005) { std::memcpy(out, pa, sizeof(pa)); return; }
        t = (lev - f0) / (f1 - f0);
        goto interpolate;
      }
    }
    if ((f1 == f0) && (pa[2] == 0.0)) t = 1.0f;
    else if (f1 == f0) t = 0.0f;
  }
interpolate:
  for (int ax = 0; ax < 3; ++ax) {
    const float d = (float)g[ax] - gc[ax];
    out[ax] = lerp_axis(d, vs[ax], oa[ax], ob[ax], t, A);
  }
}

template <class EdgeFn>
void emit_voxel(uint64_t voxel, unsigned ci, uint64_t base, uint64_t capacity, float* pos, float* norm, int cross_form,
                EdgeFn&& edge) {
  const uint64_t row = gcm::kTriRows[ci];
  const unsigned nv = kNumVerts(ci);
  (void)voxel;
  for (unsigned j = 0; j < nv; j += 3) {
    const uint64_t idx = base + j;
    float v[3][3];
    for (int m = 0; m < 3; ++m) edge((int)gcm::tri_edge(row, j + m), v[m]);
    float n[3];
    normal_of(v[0], v[1], v[2], cross_form, n);
    if (idx + 3 > capacity) continue;
    for (int m = 0; m < 3; ++m) {
      float* P = pos + 4 * (idx + m);
      float* N = norm + 4 * (idx + m);
      P[0] = v[m][0]; P[1] = v[m][1]; P[2] = v[m][2]; P[3] = 1.0f;
      N[0] = n[0]; N[1] = n[1]; N[2] = n[2]; N[3] = 0.0f;
    }
  }
}

// ---- fields ---------------------------------------------------------------------

// Euler basis rows, ZYX convention of src/Modelling.cu:401-407 (angles.x, .y, .z).
template <class T>
void euler_rows(T ax, T ay, T az, T R[9]) {
  using std::cos;
  using std::sin;
  const T sx = sin(ax), cx = cos(ax), sy = sin(ay), cy = cos(ay), sz = sin(az), cz = cos(az);
  R[0] = cz * cy; R[1] = cz * sy * sx - sz * cx; R[2] = cz * sy * cx + sz * sx;
  R[3] = sz * cy; R[4] = sz * sy * sx + cz * cx; R[5] = sz * sy * cx - cz * sx;
  R[6] = -sy;     R[7] = cy * sx;                R[8] = cy * cx;
}

inline void sincospi64(double x, double& s, double& c) {
  // Exact reduction of x to [-1, 1] half-turns before the FP64 trig.
  double r = x - 2.0 * std::nearbyint(x * 0.5);
  s = std::sin(M_PI * r);
  c = std::cos(M_PI * r);
}

// TPMS of phase (X,Y,Z) given in half-turns.  0 gyroid, 1 Schwarz-P, 2 FRD,
// 3 IWP, 5 Schwarz-D (diamond); formulas after create_lattice_kernel,
// src/lattice_files/Fft_lattice.cu:59-85, with the phase supplied by the caller.
template <class T>
T tpms_from_sc(unsigned type, T sX, T cX, T sY, T cY, T sZ, T cZ) {
  switch (type) {
    case 0: return sX * cY + sY * cZ + sZ * cX;
    case 1: return cX + cY + cZ;
    case 2: {
      const T c2X = 2 * cX * cX - 1, c2Y = 2 * cY * cY - 1, c2Z = 2 * cZ * cZ - 1;
      return 4 * (cX * cY * cZ) - (c2X * c2Y + c2Y * c2Z + c2Z * c2X);
    }
    case 3: {
      const T c2X = 2 * cX * cX - 1, c2Y = 2 * cY * cY - 1, c2Z = 2 * cZ * cZ - 1;
      return 2 * (cX * cY + cY * cZ + cZ * cX) - (c2X + c2Y + c2Z);
    }
    default: return cX * cY * cZ - sX * sY * sZ;
  }
}

struct Cell {
  int i0[3];
  float f[3];  // FP32 fractions (the discrete decisions are shared by both precisions)
  int nearest[3];
};

inline float ctrl_scale(uint32_t c, uint32_t n) {
  return (c > 1 && n > 1) ? (float)(c - 1) / (float)(n - 1) : 0.0f;
}

inline Cell locate(const uint32_t p[3], const uint32_t c[3], const float s[3]) {
  Cell k;
  for (int a = 0; a < 3; ++a) {
    const float cu = (float)p[a] * s[a];
    int i0 = (int)cu;
    if (c[a] == 1) i0 = 0;
    else if (i0 > (int)c[a] - 2) i0 = (int)c[a] - 2;
    k.i0[a] = i0;
    k.f[a] = c[a] == 1 ? 0.0f : cu - (float)i0;
    int nn = (int)(cu + 0.5f);
    if (nn > (int)c[a] - 1) nn = (int)c[a] - 1;
    k.nearest[a] = nn;
  }
  return k;
}

inline uint64_t cidx(int x, int y, int z, const uint32_t c[3]) {
  return (uint64_t)x + (uint64_t)c[0] * ((uint64_t)y + (uint64_t)c[1] * z);
}

template <class T>
T ctrl_at(const float* a, int x, int y, int z, const uint32_t c[3]) {
  return a ? (T)a[cidx(x, y, z, c)] : (T)0;
}

// Trilinear interpolation of one control array, y first, then z, then x, each
// step lerp(a, b, t) = a + t*(b - a) (FP32: fma(t, b - a, a)):
//   a(xc) = lerp(lerp(v[xc,y0,z0], v[xc,y1,z0], fy), lerp(v[xc,y0,z1], v[xc,y1,z1], fy), fz)
//   value = lerp(a(x0), a(x1), fx)
float trilinear32(const float* a, const Cell& k, const uint32_t c[3]) {
  if (!a) return 0.0f;
  const int x1 = c[0] > 1 ? k.i0[0] + 1 : 0, y1 = c[1] > 1 ? k.i0[1] + 1 : 0, z1 = c[2] > 1 ? k.i0[2] + 1 : 0;
  auto L = [](float u, float v, float t) { return std::fma(t, v - u, u); };
  const int x0 = k.i0[0], y0 = k.i0[1], z0 = k.i0[2];
  auto col = [&](int xc) {
    return L(L(a[cidx(xc, y0, z0, c)], a[cidx(xc, y1, z0, c)], k.f[1]),
             L(a[cidx(xc, y0, z1, c)], a[cidx(xc, y1, z1, c)], k.f[1]), k.f[2]);
  };
  return L(col(x0), col(x1), k.f[0]);
}

double trilinear64(const float* a, const Cell& k, const uint32_t c[3]) {
  if (!a) return 0.0;
  const int x1 = c[0] > 1 ? k.i0[0] + 1 : 0, y1 = c[1] > 1 ? k.i0[1] + 1 : 0, z1 = c[2] > 1 ? k.i0[2] + 1 : 0;
  auto L = [](double u, double v, double t) { return u + t * (v - u); };
  const int x0 = k.i0[0], y0 = k.i0[1], z0 = k.i0[2];
  const double f0 = k.f[0], f1 = k.f[1], f2 = k.f[2];
  auto col = [&](int xc) {
    return L(L(a[cidx(xc, y0, z0, c)], a[cidx(xc, y1, z0, c)], f1), L(a[cidx(xc, y0, z1, c)], a[cidx(xc, y1, z1, c)], f1),
             f2);
  };
  return L(col(x0), col(x1), f0);
}

// Phase of one lattice in half-turns: X = R q * (2 / period).
double lattice_value64(unsigned type, const double R[9], double h, const double q[3], double thick) {
  double X[3];
  for (int r = 0; r < 3; ++r) X[r] = (R[3 * r] * q[0] + R[3 * r + 1] * q[1] + R[3 * r + 2] * q[2]) * h;
  double s[3], c[3];
  for (int r = 0; r < 3; ++r) sincospi64(X[r], s[r], c[r]);
  return tpms_from_sc<double>(type, s[0], c[0], s[1], c[1], s[2], c[2]) - thick;
}

// ---- compensated FP32 arithmetic of the graded lattices ---------------------------
//
// The GPU evaluates the graded lattices with pairs of floats (hi + lo) from the
// parameter interpolation through the reduced phase, so that the phase X (up to
// ~55 half-turns at 512^3) keeps ~40 bits instead of 24.  Every step below is an
// IEEE float operation (add, sub, mul, fma, div) in a fixed order, plus double
// add/mul/div/rint on the rare path of angles outside [-3.156, 3.156]; this is a
// separate restatement of that sequence, so its results equal the kernels' bit
// for bit.  Angles go through a table of sin/cos(k/32) pairs
// (gpucadforam_gb300/csrc/angle_table.h, generated from decimal Taylor series);
// sin(pi r) and cos(pi r) of the reduced phase are their Taylor polynomials.
struct PF {
  float h, l;
};

inline PF two_sum(float a, float b) {
  const float s = a + b, bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
inline PF pf_diff(PF b, PF a) {
  const PF d = two_sum(b.h, -a.h);
  return {d.h, d.l + (b.l - a.l)};
}
// u + t * d
inline PF pf_at(PF u, PF d, float t) {
  const float p = t * d.h;
  float pe = std::fma(t, d.h, -p);
  pe = std::fma(t, d.l, pe);
  const PF s = two_sum(u.h, p);
  return {s.h, (s.l + pe) + u.l};
}
inline PF pf_lerp(PF a, PF b, float t) { return pf_at(a, pf_diff(b, a), t); }
inline PF pf_mulf(PF a, float f) {
  const float p = a.h * f;
  float pe = std::fma(a.h, f, -p);
  pe = std::fma(a.l, f, pe);
  return {p, pe};
}
inline PF pf_mul(PF a, PF b) {
  const float p = a.h * b.h;
  float pe = std::fma(a.h, b.h, -p);
  pe = std::fma(a.h, b.l, pe);
  pe = std::fma(a.l, b.h, pe);
  return {p, pe};
}
inline PF pf_add(PF a, PF b) {
  const PF s = two_sum(a.h, b.h);
  return {s.h, s.l + (a.l + b.l)};
}
inline PF pf_neg(PF a) { return {-a.h, -a.l}; }
// 2 / P
inline PF pf_two_over(PF P) {
  const float hh = 2.0f / P.h;
  float r = std::fma(-hh, P.h, 2.0f);
  r = std::fma(-hh, P.l, r);
  return {hh, r * (0.5f * hh)};
}

constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23: adding it rounds to an integer
inline int32_t fbits(float f) {
  int32_t i;
  std::memcpy(&i, &f, 4);
  return i;
}

const float kAngleTab[][4] = {GCM_ANGLE_TABLE_ROWS};

// sin and cos of the angle a (a pair) as pairs: table entry at k/32 nearest a,
// corrected by the Taylor series of the remainder (|d| <= 1/64).
inline void pf_sincos(PF a, PF& s, PF& c) {
  if (!(std::fabs(a.h) <= (float)GCM_ANGLE_K / GCM_ANGLE_STEP_INV)) {
    const double two_pi = 6.283185307179586;
    double A = (double)a.h + (double)a.l;
    const double m = std::rint(A / two_pi);
    A = A - m * two_pi;
    a.h = (float)A;
    a.l = (float)(A - (double)a.h);
  }
  const float t = std::fma(a.h, (float)GCM_ANGLE_STEP_INV, kMagic);
  const float kf = t - kMagic;
  int k = fbits(t) - fbits(kMagic);
  k = std::min(std::max(k, -GCM_ANGLE_K), GCM_ANGLE_K);
  float d = std::fma(kf, -1.0f / GCM_ANGLE_STEP_INV, a.h);
  d = d + a.l;
  const float* e = kAngleTab[k + GCM_ANGLE_K];
  const float d2 = d * d, d3 = d2 * d;
  const float sd = std::fma(d3, -0x1.555556p-3f, d);
  const float cm1 = d2 * std::fma(d2, 0x1.555556p-5f, -0.5f);
  float sl = std::fma(e[0], cm1, e[1]);
  sl = std::fma(e[2], sd, sl);
  sl = std::fma(e[3], sd, sl);
  float cl = std::fma(e[2], cm1, e[3]);
  cl = std::fma(-e[0], sd, cl);
  cl = std::fma(-e[1], sd, cl);
  // renormalised, so that products drop only terms of order lo * lo
  s = two_sum(e[0], sl);
  c = two_sum(e[2], cl);
}

// X mod 2 (half-turns) as one float.
inline float pf_reduce(PF X) {
  const float t = std::fma(X.h, 0.5f, kMagic);
  const float kf = t - kMagic;
  const float r = std::fma(kf, -2.0f, X.h);
  return r + X.l;
}

// sin(pi r), cos(pi r): quarter-turn j = rint(2r), u = r - j/2, Taylor polynomials in u.
inline void sincospi_taylor(float r, float& s, float& c) {
  const float t = std::fma(r, 2.0f, kMagic);
  const float jf = t - kMagic;
  const int j = fbits(t) & 3;
  const float u = std::fma(jf, -0.5f, r);
  const float z = u * u;
  float ps = std::fma(z, GCM_SINPI_C9, GCM_SINPI_C7);
  ps = std::fma(z, ps, GCM_SINPI_C5);
  ps = std::fma(z, ps, GCM_SINPI_C3);
  ps = std::fma(z, ps, GCM_SINPI_C1);
  const float sn = u * ps;
  float pc = std::fma(z, GCM_COSPI_C10, GCM_COSPI_C8);
  pc = std::fma(z, pc, GCM_COSPI_C6);
  pc = std::fma(z, pc, GCM_COSPI_C4);
  pc = std::fma(z, pc, GCM_COSPI_C2);
  const float cs = std::fma(z, pc, 1.0f);
  switch (j) {
    case 0: s = sn; c = cs; break;
    case 1: s = cs; c = -sn; break;
    case 2: s = -sn; c = -cs; break;
    default: s = -cs; c = sn; break;
  }
}

inline float tpms_of_phase(unsigned type, const float r[3], float thick) {
  float s[3], c[3];
  for (int k = 0; k < 3; ++k) sincospi_taylor(r[k], s[k], c[k]);
  return tpms_from_sc<float>(type, s[0], c[0], s[1], c[1], s[2], c[2]) - thick;
}

// PARAMS mode: one parameter's compensated trilinear value, y first, then z,
// then x (as trilinear64), with the x step as record + fraction.
PF trilinear_pf(const float* a, const Cell& k, const uint32_t c[3]) {
  if (!a) return {0.0f, 0.0f};
  const int x1 = c[0] > 1 ? k.i0[0] + 1 : 0, y1 = c[1] > 1 ? k.i0[1] + 1 : 0, z1 = c[2] > 1 ? k.i0[2] + 1 : 0;
  const int y0 = k.i0[1], z0 = k.i0[2];
  auto col = [&](int xc) {
    const PF A = pf_lerp({a[cidx(xc, y0, z0, c)], 0.0f}, {a[cidx(xc, y1, z0, c)], 0.0f}, k.f[1]);
    const PF B = pf_lerp({a[cidx(xc, y0, z1, c)], 0.0f}, {a[cidx(xc, y1, z1, c)], 0.0f}, k.f[1]);
    return pf_lerp(A, B, k.f[2]);
  };
  return pf_lerp(col(k.i0[0]), col(x1), k.f[0]);
}

// PARAMS mode phase: q rotated by Rx, Ry, Rz in turn (the rows of Modelling.cu:
// 401-407 applied one axis at a time), scaled by 2/P, reduced mod 2.
void params_phase(PF P, PF ax, PF ay, PF az, const float q[3], float r[3]) {
  PF sx, cx, sy, cy, sz, cz;
  pf_sincos(ax, sx, cx);
  pf_sincos(ay, sy, cy);
  pf_sincos(az, sz, cz);
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

// BLEND mode per control point: M = R * (2 / period) in double from the table's
// sin/cos pairs, each entry split into a float pair (row-major M[r][j]).
void blend_matrix(float ax, float ay, float az, float period, PF M[9]) {
  PF s[3], c[3];
  pf_sincos({ax, 0.0f}, s[0], c[0]);
  pf_sincos({ay, 0.0f}, s[1], c[1]);
  pf_sincos({az, 0.0f}, s[2], c[2]);
  const double sx = (double)s[0].h + (double)s[0].l, cx = (double)c[0].h + (double)c[0].l;
  const double sy = (double)s[1].h + (double)s[1].l, cy = (double)c[1].h + (double)c[1].l;
  const double sz = (double)s[2].h + (double)s[2].l, cz = (double)c[2].h + (double)c[2].l;
  double R[9];
  R[0] = cz * cy; R[1] = (cz * sy) * sx - sz * cx; R[2] = (cz * sy) * cx + sz * sx;
  R[3] = sz * cy; R[4] = (sz * sy) * sx + cz * cx; R[5] = (sz * sy) * cx - cz * sx;
  R[6] = -sy;     R[7] = cy * sx;                  R[8] = cy * cx;
  const double H = 2.0 / (double)period;
  for (int i = 0; i < 9; ++i) {
    const double m = R[i] * H;
    M[i].h = (float)m;
    M[i].l = (float)(m - (double)M[i].h);
  }
}

// BLEND mode phase of one corner lattice: X_r = M_r0 q0 + (M_r1 q1 + M_r2 q2).
void blend_phase(const PF M[9], const float q[3], float r[3]) {
  for (int i = 0; i < 3; ++i) {
    const PF K = pf_add(pf_mulf(M[3 * i + 1], q[1]), pf_mulf(M[3 * i + 2], q[2]));
    r[i] = pf_reduce(pf_add(pf_mulf(M[3 * i], q[0]), K));
  }
}

template <bool F64, class Out>
void lattice_field_impl(const orc_lattice* L, uint32_t nx, uint32_t ny, uint32_t nz, Out* out, int threads,
                        uint32_t z0 = 0, uint32_t nplanes = 0) {
  const uint32_t c[3] = {L->cx, L->cy, L->cz};
  const uint32_t n[3] = {nx, ny, nz};
  const float s[3] = {ctrl_scale(c[0], nx), ctrl_scale(c[1], ny), ctrl_scale(c[2], nz)};
  const uint64_t nctrl = (uint64_t)c[0] * c[1] * c[2];
  // Per-control-point rotation rows (blend mode), from the control Euler angles.
  std::vector<PF> M32(9 * nctrl);
  std::vector<double> R64(9 * nctrl);
  for (uint64_t i = 0; i < nctrl; ++i) {
    const float ax = L->euler ? L->euler[i] : 0.f, ay = L->euler ? L->euler[nctrl + i] : 0.f,
                az = L->euler ? L->euler[2 * nctrl + i] : 0.f;
    if (L->mode == 1) blend_matrix(ax, ay, az, L->period[i], &M32[9 * i]);
    euler_rows<double>(ax, ay, az, &R64[9 * i]);
  }
  const int nt = set_threads(threads);
  if (nplanes == 0) nplanes = nz - z0;
  const uint64_t plane = (uint64_t)nx * ny;
  const uint64_t total = plane * nplanes;
#pragma omp parallel for schedule(static) num_threads(nt)
  for (int64_t ii = 0; ii < (int64_t)total; ++ii) {
    const uint64_t i = (uint64_t)ii;
    const uint32_t p[3] = {(uint32_t)(i % nx), (uint32_t)((i / nx) % ny), (uint32_t)(i / plane) + z0};
    const Cell k = locate(p, c, s);
    if (L->mode == 0) {
      const uint64_t ni = cidx(k.nearest[0], k.nearest[1], k.nearest[2], c);
      const unsigned type = L->type[ni];
      if (!F64) {
        const PF P = trilinear_pf(L->period, k, c);
        const PF ax = trilinear_pf(L->euler, k, c);
        const PF ay = trilinear_pf(L->euler ? L->euler + nctrl : nullptr, k, c);
        const PF az = trilinear_pf(L->euler ? L->euler + 2 * nctrl : nullptr, k, c);
        const float th = trilinear32(L->thickness, k, c);
        const float q[3] = {(float)p[0] - L->origin[0], (float)p[1] - L->origin[1], (float)p[2] - L->origin[2]};
        float r[3];
        params_phase(P, ax, ay, az, q, r);
        out[i] = (Out)tpms_of_phase(type, r, th);
      } else {
        const double P = trilinear64(L->period, k, c);
        const double ax = trilinear64(L->euler, k, c);
        const double ay = trilinear64(L->euler ? L->euler + nctrl : nullptr, k, c);
        const double az = trilinear64(L->euler ? L->euler + 2 * nctrl : nullptr, k, c);
        const double th = trilinear64(L->thickness, k, c);
        double R[9];
        euler_rows<double>(ax, ay, az, R);
        const double q[3] = {(double)p[0] - (double)L->origin[0], (double)p[1] - (double)L->origin[1],
                             (double)p[2] - (double)L->origin[2]};
        out[i] = (Out)lattice_value64(type, R, 2.0 / P, q, th);
      }
    } else {
      // Blend: every control point anchors its own uniform lattice at its position;
      // the field is the trilinear blend of the 8 surrounding lattices.
      if (!F64) {
        float acc = 0.0f;
        for (int corner = 0; corner < 8; ++corner) {
          const int d[3] = {corner & 1, (corner >> 1) & 1, (corner >> 2) & 1};
          int g[3];
          float wa[3], q[3];
          for (int a = 0; a < 3; ++a) {
            g[a] = c[a] > 1 ? k.i0[a] + d[a] : 0;
            wa[a] = (c[a] > 1) ? (d[a] ? k.f[a] : 1.0f - k.f[a]) : (d[a] ? 0.0f : 1.0f);
            const float anchor = c[a] > 1 ? (float)g[a] * ((float)(n[a] - 1) / (float)(c[a] - 1)) : 0.0f;
            q[a] = (float)p[a] - anchor;
          }
          const float w = wa[0] * (wa[1] * wa[2]);
          if (w == 0.0f) continue;
          const uint64_t ci = cidx(g[0], g[1], g[2], c);
          float r[3];
          blend_phase(&M32[9 * ci], q, r);
          const float v = tpms_of_phase(L->type[ci], r, L->thickness ? L->thickness[ci] : 0.0f);
          acc = std::fma(w, v, acc);
        }
        out[i] = (Out)acc;
      } else {
        double acc = 0.0;
        for (int corner = 0; corner < 8; ++corner) {
          const int d[3] = {corner & 1, (corner >> 1) & 1, (corner >> 2) & 1};
          int g[3];
          double wa[3], q[3];
          for (int a = 0; a < 3; ++a) {
            g[a] = c[a] > 1 ? k.i0[a] + d[a] : 0;
            wa[a] = (c[a] > 1) ? (d[a] ? (double)k.f[a] : 1.0 - (double)k.f[a]) : (d[a] ? 0.0 : 1.0);
            // the anchor positions are FP32 numbers (a modelling decision shared by
            // both precisions, like the cell fractions)
            const double anchor = c[a] > 1 ? (double)((float)g[a] * ((float)(n[a] - 1) / (float)(c[a] - 1))) : 0.0;
            q[a] = (double)p[a] - anchor;
          }
          const double w = wa[0] * (wa[1] * wa[2]);
          if (w == 0.0) continue;
          const uint64_t ci = cidx(g[0], g[1], g[2], c);
          acc += w * lattice_value64(L->type[ci], &R64[9 * ci], 2.0 / (double)L->period[ci], q,
                                     L->thickness ? L->thickness[ci] : 0.0);
        }
        out[i] = (Out)acc;
      }
    }
  }
}

// ---- primitives (src/Modelling.cu) -----------------------------------------------------

template <class T>
T sq(T x) { return x * x; }

// Field of one primitive at a point given in the scene frame.  Float promotions
// follow the reference kernels (literals such as 2.0 promote to double).
template <class T>
T primitive_at(uint32_t kind, uint32_t flag, const float* center, const float* v3, const float* p, T X, T Y, T Z) {
  using std::fabs;
  using std::sqrt;
  const T cxv = center[0], cyv = center[1], czv = center[2];
  switch (kind) {
    case 0: {  // implicit_sphere_kernel :314-361
      const T x = X - cxv, y = Y - cyv, z = Z - czv;
      const T r = p[0], t = (T)(p[1] / 2.0);
      const T d2 = sq(x) + sq(y) + sq(z);
      if (flag) {
        const T f1 = d2 - sq(r - t), f2 = d2 - sq(r + t);
        return (T)std::max((double)(f1 * -1.0), (double)f2);
      }
      return d2 - sq(r);
    }
    case 1: {  // distance_from_line_kernel :244-302 (capped cylinder / disc)
      const T r = p[0], td = (T)(p[1] / 2.0), tda = (T)(p[2] / 2.0);
      const T am = sqrt(sq((T)v3[0]) + sq((T)v3[1]) + sq((T)v3[2]));
      const T ax = v3[0] / am, ay = v3[1] / am, az = v3[2] / am;
      const T ex = ax + cxv, ey = ay + cyv, ez = az + czv;
      const T w1x = X - cxv, w1y = Y - cyv, w1z = Z - czv;
      const T w2x = X - ex, w2y = Y - ey, w2z = Z - ez;
      const T w3x = ex - cxv, w3y = ey - cyv, w3z = ez - czv;
      const T dx = w1y * w2z - w1z * w2y, dy = w1z * w2x - w1x * w2z, dz = w1x * w2y - w1y * w2x;
      const T e = sqrt(sq(dx) + sq(dy) + sq(dz));
      const T dis = sqrt(sq(w3x) + sq(w3y) + sq(w3z));
      const T f = e / dis;
      const T g = (X - cxv) * ax + (Y - cyv) * ay + (Z - czv) * az;
      const T fld1 = std::max(g - tda, (g + tda) * (T)-1);
      T fld2;
      if (flag) fld2 = (T)std::max((double)(f - (r + td)), (double)(f - (r - td)) * -1.0);
      else fld2 = f - r;
      return std::max(fld1, fld2);
    }
    default: {
      const T x = X - cxv, y = Y - cyv, z = Z - czv;
      T R[9];
      euler_rows<T>((T)v3[0], (T)v3[1], (T)v3[2], R);
      const T a = x * R[0] + y * R[1] + z * R[2];
      const T b = x * R[3] + y * R[4] + z * R[5];
      const T c = x * R[6] + y * R[7] + z * R[8];
      switch (kind) {
        case 2: {  // implicit_cuboid_kernel :375-421
          const T wx = (T)(p[0] / 2.0), wy = (T)(p[1] / 2.0), wz = (T)(p[2] / 2.0);
          return std::max(std::max(fabs(a) - wx, fabs(b) - wy), fabs(c) - wz);
        }
        case 3: {  // implicit_cuboid_shell_kernel :435-487
          const T wx = (T)(p[0] / 2.0), wy = (T)(p[1] / 2.0), wz = (T)(p[2] / 2.0), th = p[3];
          const T f11 = fabs(a) - wx, f12 = fabs(a) - (wx - th);
          const T f21 = fabs(b) - wy, f22 = fabs(b) - (wy - th);
          const T f3 = fabs(c) - wz;
          const T inner = (T)((double)std::max(f12, f22) * -1.0);
          return std::max(std::max(std::max(f11, f21), inner), f3);
        }
        case 4: {  // implicit_torus_kernel :569-616
          const T side = (T)p[0] - sqrt(sq(a) + sq(b));
          return sq(c) - sq((T)p[1]) + sq(side);
        }
        case 5: {  // implicit_cone_kernel :631-683
          const T br = p[0], hgt = p[1];
          const T k2 = sq(hgt / br);
          const T g = (T)(b - hgt / 2.0);
          const T h = (T)std::max((double)(g - hgt / 2.0) * 100, (double)(g + hgt / 2.0) * 100 * -1.0);
          const T f1 = ((sq(a) + sq(c)) * k2) - sq(b - hgt);
          return std::max(f1, h);
        }
        case 6: {  // implicit_cone_frustum_kernel :698-750
          const T tr = p[0], br = p[1], hgt = p[2];
          const T rd = ((hgt - b) / hgt) * (br - tr);
          const T g = (T)(b - hgt / 2.0);
          const T h = (T)std::max((double)(g - hgt / 2.0) * 100, (double)(g + hgt / 2.0) * 100 * -1.0);
          const T f1 = (T)((double)(sq(a) + sq(c)) - sq((double)(rd + tr)));
          return std::max(f1, h);
        }
        default: {  // 7: implicit_pyramid_frustum_kernel :501-557
          const T xwb = (T)(p[0] / 2.0), xwt = (T)(p[1] / 2.0), yh = p[2];
          const T zwb = (T)(p[3] / 2.0), zwt = (T)(p[4] / 2.0);
          const T ratio = (yh - b) / yh;
          const T xw = (ratio * (xwb - xwt)) + xwt;
          const T f1 = fabs(a) - xw;
          const T f2 = (T)(fabs(b - yh / 2) - yh / 2);
          const T zw = (ratio * (zwb - zwt)) + zwt;
          const T f3 = fabs(c) - zw;
          return std::max(std::max(f1, f2), f3);
        }
      }
    }
  }
}

// The float primitive fields as the GPU evaluates them by default: sample
// offset t = index - origin and spacing sp per axis; the reference build's
// operation order and fused multiply-adds (position t * sp - c fused, sums of
// products and cross products fusing their first product, lerps of the
// pyramid widths fused, cone height terms in double) with correctly rounded
// squares where the reference calls powf(v, 2).  The basis rows come from the
// host's sinf/cosf, so rotated kinds agree with the GPU (CUDA sinf/cosf) only
// to the trig's last bits.
float primitive_f32(uint32_t kind, uint32_t flag, const float* c, const float* v3, const float* p, const float t[3],
                    const float sp[3]) {
  using std::fma;
  auto sqr = [](float v) { return v * v; };
  switch (kind) {
    case 0: {
      const float x = fma(t[0], sp[0], -c[0]), y = fma(t[1], sp[1], -c[1]), z = fma(t[2], sp[2], -c[2]);
      const float r = p[0], td = p[1] * 0.5f;
      const float d2 = (sqr(x) + sqr(y)) + sqr(z);
      if (flag) return std::fmax(-(d2 - sqr(r - td)), d2 - sqr(r + td));
      return d2 - sqr(r);
    }
    case 1: {
      const float r = p[0], td = p[1] * 0.5f, tda = p[2] * 0.5f;
      const float am = std::sqrt((sqr(v3[0]) + sqr(v3[1])) + sqr(v3[2]));
      float ax[3], end[3], w1[3], w2[3], w3[3];
      for (int k = 0; k < 3; ++k) {
        ax[k] = v3[k] / am;
        end[k] = ax[k] + c[k];
      }
      for (int k = 0; k < 3; ++k) {
        w1[k] = fma(t[k], sp[k], -c[k]);
        w2[k] = fma(t[k], sp[k], -end[k]);
        w3[k] = end[k] - c[k];
      }
      const float dis = std::sqrt((sqr(w3[0]) + sqr(w3[1])) + sqr(w3[2]));
      const float dx = fma(w1[1], w2[2], -(w1[2] * w2[1])), dy = fma(w1[2], w2[0], -(w1[0] * w2[2])),
                  dz = fma(w1[0], w2[1], -(w1[1] * w2[0]));
      const float f = std::sqrt((sqr(dx) + sqr(dy)) + sqr(dz)) / dis;
      const float g = fma(w1[2], ax[2], fma(w1[0], ax[0], w1[1] * ax[1]));
      const float fld1 = std::fmax(g - tda, -(g + tda));
      const float fld2 = flag ? std::fmax(f - (r + td), -(f - (r - td))) : f - r;
      return std::fmax(fld1, fld2);
    }
    default: {
      const float x = fma(t[0], sp[0], -c[0]), y = fma(t[1], sp[1], -c[1]), z = fma(t[2], sp[2], -c[2]);
      const float ax = v3[0], ay = v3[1], az = v3[2];
      const float sx = std::sin(ax), cx = std::cos(ax), sy = std::sin(ay), cy = std::cos(ay), sz = std::sin(az),
                  cz = std::cos(az);
      const float R0 = cz * cy, R1 = fma(cz * sy, sx, -(sz * cx)), R2 = fma(cz * sy, cx, sz * sx);
      const float R3 = sz * cy, R4 = fma(sz * sy, sx, cz * cx), R5 = fma(sz * sy, cx, -(cz * sx));
      const float R7 = cy * sx, R8 = cy * cx;
      const float a = fma(z, R2, fma(x, R0, y * R1));
      const float b = fma(z, R5, fma(x, R3, y * R4));
      const float cc = fma(z, R8, fma(y, R7, -(x * sy)));
      auto slab = [](float bb, float h) {
        const float g = (float)((double)bb - (double)h / 2.0);
        return (float)std::fmax(((double)g - (double)h / 2.0) * 100.0, -(((double)g + (double)h / 2.0) * 100.0));
      };
      switch (kind) {
        case 2:
          return std::fmax(std::fmax(std::fabs(a) - p[0] * 0.5f, std::fabs(b) - p[1] * 0.5f),
                           std::fabs(cc) - p[2] * 0.5f);
        case 3: {
          const float wx = p[0] * 0.5f, wy = p[1] * 0.5f, wz = p[2] * 0.5f, th = p[3];
          const float f11 = std::fabs(a) - wx, f12 = std::fabs(a) - (wx - th);
          const float f21 = std::fabs(b) - wy, f22 = std::fabs(b) - (wy - th);
          return std::fmax(std::fmax(std::fmax(f11, f21), -std::fmax(f12, f22)), std::fabs(cc) - wz);
        }
        case 4: {
          const float side = p[0] - std::sqrt(sqr(a) + sqr(b));
          return (sqr(cc) - sqr(p[1])) + sqr(side);
        }
        case 5: {
          const float k2 = sqr(p[1] / p[0]);
          return std::fmax(fma(sqr(a) + sqr(cc), k2, -sqr(b - p[1])), slab(b, p[1]));
        }
        case 6: {
          const float tr = p[0], br = p[1], h = p[2];
          const float rr = fma((h - b) / h, br - tr, tr);
          const float f1 = (float)((double)(sqr(a) + sqr(cc)) - (double)rr * (double)rr);
          return std::fmax(f1, slab(b, h));
        }
        default: {
          const float xwb = p[0] * 0.5f, xwt = p[1] * 0.5f, yh = p[2], zwb = p[3] * 0.5f, zwt = p[4] * 0.5f;
          const float ratio = (yh - b) / yh, hy = yh * 0.5f;
          const float f1 = std::fabs(a) - fma(ratio, xwb - xwt, xwt);
          const float f2 = std::fabs(b - hy) - hy;
          const float f3 = std::fabs(cc) - fma(ratio, zwb - zwt, zwt);
          return std::fmax(std::fmax(f1, f2), f3);
        }
      }
    }
  }
}

template <class T>
T csg_apply(T f, T g, uint32_t op) {
  switch (op) {
    case 1: return std::max(f, -g);
    case 2: return std::max(f, g);
    default: return std::min(f, g);
  }
}

// CSG scene: coordinates x = (i - origin) * spacing in the scene frame; the
// primitive formulas are those of src/Modelling.cu; the combination is a running
// min / max(f, -g) / max over the list, starting from +inf.
template <class T, class Out>
void csg_impl(const orc_prim* prims, uint32_t n, const float* origin, const float* spacing, uint32_t nx,
                     uint32_t ny, uint32_t nz, Out* out, int threads) {
  const int nt = set_threads(threads);
  const uint64_t total = (uint64_t)nx * ny * nz;
#pragma omp parallel for schedule(static) num_threads(nt)
  for (int64_t ii = 0; ii < (int64_t)total; ++ii) {
    const uint64_t i = (uint64_t)ii;
    const uint32_t px = (uint32_t)(i % nx), py = (uint32_t)((i / nx) % ny), pz = (uint32_t)(i / ((uint64_t)nx * ny));
    const float t[3] = {(float)px - origin[0], (float)py - origin[1], (float)pz - origin[2]};
    T f = std::numeric_limits<T>::infinity();
    for (uint32_t k = 0; k < n; ++k) {
      const orc_prim& P = prims[k];
      T g;
      if constexpr (sizeof(T) == 4) {
        g = primitive_f32(P.kind, P.flag, P.center, P.v3, P.p, t, spacing);
      } else {
        g = primitive_at<T>(P.kind, P.flag, P.center, P.v3, P.p, (T)t[0] * (T)spacing[0], (T)t[1] * (T)spacing[1],
                            (T)t[2] * (T)spacing[2]);
      }
      f = csg_apply<T>(f, g, P.op);
    }
    out[i] = (Out)f;
  }
}

}  // namespace

extern "C" {

// Pattern of the reference kernels as nvcc builds them (pinned by
// tests/golden/golden_mc.npz): corners p + vs (no fusion), edge delta b - a,
// lerp fma(t, b - a, a), cross terms fma(a, b, -(c*d)).
uint32_t orc_default_arith(void) { return 4u | (1u << 4); }

void orc_mc_classify(const float* field, uint32_t nx, uint32_t ny, uint32_t nz, float iso, uint32_t* voxel_verts,
                     uint32_t* voxel_occupied, uint8_t* cube) {
  const uint64_t nv = (uint64_t)(nx - 1) * (ny - 1) * (nz - 1);
#pragma omp parallel for schedule(static)
  for (int64_t vv = 0; vv < (int64_t)nv; ++vv) {
    uint32_t x, y, z;
    voxel_pos((uint64_t)vv, nx, ny, x, y, z);
    float c[8];
    corners(field, x, y, z, nx, ny, c);
    const unsigned ci = cube_index(c, iso);
    const unsigned n = kNumVerts(ci);
    if (voxel_verts) voxel_verts[vv] = n;
    if (voxel_occupied) voxel_occupied[vv] = n > 0;
    if (cube) cube[vv] = (uint8_t)ci;
  }
}

// thrust::exclusive_scan over uint (src/MarchingCubes_kernel.cu:3198-3203): 32-bit
// wrap-around sums; the 64-bit total is returned.
uint64_t orc_scan_exclusive_u32(const uint32_t* in, uint32_t* out, uint64_t n) {
  uint64_t acc = 0;
  for (uint64_t i = 0; i < n; ++i) {
    out[i] = (uint32_t)acc;
    acc += in[i];
  }
  return acc;
}

// compactVoxels (src/MarchingCubes_kernel.cu:1594-1608).
void orc_mc_compact(const uint32_t* occ, const uint32_t* occ_scan, uint64_t n, uint32_t* out) {
  for (uint64_t i = 0; i < n; ++i)
    if (occ[i]) out[occ_scan[i]] = (uint32_t)i;
}

// generateTriangles_lattice_kernel_3 (src/MarchingCubes_kernel.cu:3041-3170) with
// the classify cube index; a triangle is written only when all three of its
// vertices fit below capacity_verts.
void orc_mc_generate(const float* field, uint32_t nx, uint32_t ny, uint32_t nz, const float* vs, const float* gc,
                     float iso, const uint32_t* compacted, uint64_t active, const uint32_t* verts_scan,
                     uint64_t capacity, float* pos, float* norm, uint32_t arith) {
  (void)nz;
  const Arith A = decode(arith);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t a = 0; a < (int64_t)active; ++a) {
    const uint64_t voxel = compacted[a];
    uint32_t g[3];
    voxel_pos(voxel, nx, ny, g[0], g[1], g[2]);
    float c[8];
    corners(field, g[0], g[1], g[2], nx, ny, c);
    const unsigned ci = cube_index(c, iso);
    emit_voxel(voxel, ci, verts_scan[voxel], capacity, pos, norm, A.cross,
               [&](int e, float* out) { edge_point_plain(g, vs, gc, e, c, iso, A, out); });
  }
}

// generateTriangles_lattice_kernel_newone (src/MarchingCubes_kernel.cu:3678-3817):
// cube index from the label field, vertices from the normalised field.
void orc_mc_generate_band(const float* label, const float* nf, uint32_t nx, uint32_t ny, uint32_t nz, const float* vs,
                          const float* gc, float iso, float lo, float hi, const uint32_t* compacted, uint64_t active,
                          const uint32_t* verts_scan, uint64_t capacity, float* pos, float* norm, uint32_t arith) {
  (void)nz;
  const Arith A = decode(arith);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t a = 0; a < (int64_t)active; ++a) {
    const uint64_t voxel = compacted[a];
    uint32_t g[3];
    voxel_pos(voxel, nx, ny, g[0], g[1], g[2]);
    float lab[8], fv[8];
    corners(label, g[0], g[1], g[2], nx, ny, lab);
    corners(nf, g[0], g[1], g[2], nx, ny, fv);
    const unsigned ci = cube_index(lab, iso);
    emit_voxel(voxel, ci, verts_scan[voxel], capacity, pos, norm, A.cross,
               [&](int e, float* out) { edge_point_band(g, vs, gc, e, lab, fv, lo, hi, A, out); });
  }
}

uint64_t orc_mesh_field(const float* field, uint32_t nx, uint32_t ny, uint32_t nz, const float* vs, const float* gc,
                        float iso, float* pos, float* norm, uint64_t capacity, uint64_t* active_out, int threads) {
  const uint64_t nv = (uint64_t)(nx - 1) * (ny - 1) * (nz - 1);
  const int nt = set_threads(threads);
  std::vector<uint32_t> verts(nv);
#pragma omp parallel for schedule(static) num_threads(nt)
  for (int64_t vv = 0; vv < (int64_t)nv; ++vv) {
    uint32_t x, y, z;
    voxel_pos((uint64_t)vv, nx, ny, x, y, z);
    float c[8];
    corners(field, x, y, z, nx, ny, c);
    verts[vv] = kNumVerts(cube_index(c, iso));
  }
  // Two-level exclusive scan over the per-voxel counts.
  std::vector<uint64_t> chunk_sum(nt + 1, 0), chunk_act(nt + 1, 0);
  std::vector<uint64_t> scan(nv);
#pragma omp parallel num_threads(nt)
  {
#ifdef _OPENMP
    const int t = omp_get_thread_num(), T = omp_get_num_threads();
#else
    const int t = 0, T = 1;
#endif
    const uint64_t b = nv * t / T, e = nv * (t + 1) / T;
    uint64_t s = 0, a = 0;
    for (uint64_t i = b; i < e; ++i) { s += verts[i]; a += verts[i] > 0; }
    chunk_sum[t + 1] = s;
    chunk_act[t + 1] = a;
#pragma omp barrier
#pragma omp single
    for (int i = 1; i <= T; ++i) { chunk_sum[i] += chunk_sum[i - 1]; chunk_act[i] += chunk_act[i - 1]; }
    uint64_t acc = chunk_sum[t];
    for (uint64_t i = b; i < e; ++i) { scan[i] = acc; acc += verts[i]; }
  }
  const uint64_t total = chunk_sum[nt];
  if (active_out) *active_out = chunk_act[nt];
  const Arith A = decode(orc_default_arith());
#pragma omp parallel for schedule(dynamic, 4096) num_threads(nt)
  for (int64_t vv = 0; vv < (int64_t)nv; ++vv) {
    if (!verts[vv]) continue;
    uint32_t g[3];
    voxel_pos((uint64_t)vv, nx, ny, g[0], g[1], g[2]);
    float c[8];
    corners(field, g[0], g[1], g[2], nx, ny, c);
    const unsigned ci = cube_index(c, iso);
    emit_voxel((uint64_t)vv, ci, scan[vv], capacity, pos, norm, A.cross,
               [&](int e, float* out) { edge_point_plain(g, vs, gc, e, c, iso, A, out); });
  }
  return total;
}

// ---- retained CSG accumulation ---------------------------------------------------

// classify_copy_Voxel, static mode (src/MarchingCubes_kernel.cu:158-447), as
// Isosurface::copy_parameter launches it (src/Isosurface.cu:16-27): samples
// 0 .. P-2 (the launch bound excludes the last one); the new sign from the
// boolean of f and the old sign; on each +x, +y, +z edge that f crosses the
// fraction (iso - v) / (w - v) replaces a non-positive stored fraction or is
// averaged with a positive one, (t_old + t) * 0.5 in double.
void orc_csg_retain(orc_csg_point* acc, const float* f, uint32_t nx, uint32_t ny, uint32_t nz, float iso,
                    uint32_t op) {
  const uint64_t plane = (uint64_t)nx * ny, total = plane * nz;
  for (uint64_t i = 0; i + 1 < total; ++i) {
    const uint32_t x = (uint32_t)(i % nx), y = (uint32_t)((i / nx) % ny), z = (uint32_t)(i / plane);
    orc_csg_point pt = acc[i];
    const float v = f[i];
    bool inside;
    if (op == 1) inside = (v >= iso) && ((float)pt.val < iso);
    else if (op == 2) inside = (v < iso) && ((float)pt.val < iso);
    else inside = (v < iso) || ((float)pt.val < iso);
    pt.val = inside ? -1 : 1;
    const uint64_t stride[3] = {1, nx, plane};
    const bool has[3] = {x + 1 < nx, y + 1 < ny, z + 1 < nz};
    for (int a = 0; a < 3; ++a) {
      if (!has[a]) continue;
      const float w = f[i + stride[a]];
      if ((w < iso && v >= iso) || (w >= iso && v < iso)) {
        const float t = (iso - v) / (w - v);
        pt.t[a] = pt.t[a] > 0 ? (float)((double)(pt.t[a] + t) * 0.5) : t;
      }
    }
    acc[i] = pt;
  }
}

// classify_copy_Voxel, lattice-band ("dynamic") mode (src/MarchingCubes_kernel.cu:
// 158-447 with dynamic = true; its `fixed` flag is not read): the object is the
// open band iso1 < L < iso2 of the lattice field L.  Union: band or old inside;
// difference: band and old outside (the kernel's own pairing, :206-215);
// intersection: band and old inside.  On each +x, +y, +z edge the fraction is
// taken where L crosses iso1, else where it crosses iso2 (the same crossing
// test and fraction as the static mode, per band edge), and replaces or is
// averaged with the stored one.
void orc_csg_retain_band(orc_csg_point* acc, const float* lat, uint32_t nx, uint32_t ny, uint32_t nz, float iso,
                         float iso1, float iso2, uint32_t op) {
  const uint64_t plane = (uint64_t)nx * ny, total = plane * nz;
  for (uint64_t i = 0; i + 1 < total; ++i) {
    const uint32_t x = (uint32_t)(i % nx), y = (uint32_t)((i / nx) % ny), z = (uint32_t)(i / plane);
    orc_csg_point pt = acc[i];
    const float v = lat[i];
    const bool band = (v > iso1) && (v < iso2);
    bool inside;
    if (op == 1) inside = band && ((float)pt.val >= iso);
    else if (op == 2) inside = band && ((float)pt.val < iso);
    else inside = band || ((float)pt.val < iso);
    pt.val = inside ? -1 : 1;
    const uint64_t stride[3] = {1, nx, plane};
    const bool has[3] = {x + 1 < nx, y + 1 < ny, z + 1 < nz};
    for (int a = 0; a < 3; ++a) {
      if (!has[a]) continue;
      const float w = lat[i + stride[a]];
      auto crosses = [&](float lev) { return (w < lev && v >= lev) || (w >= lev && v < lev); };
      float lev;
      if (crosses(iso1)) lev = iso1;
      else if (crosses(iso2)) lev = iso2;
      else continue;
      const float t = (lev - v) / (w - v);
      pt.t[a] = pt.t[a] > 0 ? (float)((double)(pt.t[a] + t) * 0.5) : t;
    }
    acc[i] = pt;
  }
}

// Meshes of the accumulator: classifyVoxel and generateTriangles_lattice_kernel
// (src/MarchingCubes_kernel.cu:869-1052, 1865-2200) in their make_region mode
// (field == NULL) and their plain primitive mode (fixed = dynamic = false): the
// corner test, the edge running from its lower corner, the vertex at the stored
// fraction or at vertexInterp_primitive's average (:1640-1672), the normal
// calcNormal(v0, v2, v1) with w = 0.5.
uint64_t orc_mesh_retained(const orc_csg_point* acc, const float* g, uint32_t op, uint32_t nx, uint32_t ny,
                           uint32_t nz, const float* vs, const float* gc, float iso, float* pos, float* norm,
                           uint64_t capacity, uint64_t* active_out) {
  const uint64_t nvox = (uint64_t)(nx - 1) * (ny - 1) * (nz - 1);
  auto inside = [&](uint64_t i) {
    const bool a = (float)acc[i].val < iso;
    if (!g) return a;
    if (op == 1) return (g[i] >= iso) && a;
    if (op == 2) return a && (g[i] < iso);
    return a || (g[i] < iso);
  };
  auto cube = [&](uint32_t x, uint32_t y, uint32_t z) {
    unsigned ci = 0;
    for (int k = 0; k < 8; ++k)
      ci |= (unsigned)inside(pidx(x + gcm::kCornerX[k], y + gcm::kCornerY[k], z + gcm::kCornerZ[k], nx, ny)) << k;
    return ci;
  };
  std::vector<uint64_t> scan(nvox);
  uint64_t total = 0, active = 0;
  for (uint64_t v = 0; v < nvox; ++v) {
    uint32_t x, y, z;
    voxel_pos(v, nx, ny, x, y, z);
    const unsigned n = kNumVerts(cube(x, y, z));
    scan[v] = total;
    total += n;
    active += n > 0;
  }
  if (active_out) *active_out = active;
  const Arith A = decode(orc_default_arith());
  for (uint64_t v = 0; v < nvox; ++v) {
    uint32_t gp[3];
    voxel_pos(v, nx, ny, gp[0], gp[1], gp[2]);
    const unsigned ci = cube(gp[0], gp[1], gp[2]);
    const uint64_t row = gcm::kTriRows[ci];
    const unsigned nv = kNumVerts(ci);
    for (unsigned j = 0; j < nv; j += 3) {
      float vv[3][3];
      for (int m = 0; m < 3; ++m) {
        const int e = (int)gcm::tri_edge(row, j + m);
        int lo = gcm::kEdgeA[e], up = gcm::kEdgeB[e];
        const int olo[3] = {gcm::kCornerX[lo], gcm::kCornerY[lo], gcm::kCornerZ[lo]};
        const int oup[3] = {gcm::kCornerX[up], gcm::kCornerY[up], gcm::kCornerZ[up]};
        int axis = 0;
        for (int a = 0; a < 3; ++a)
          if (olo[a] != oup[a]) axis = a;
        if (olo[axis] > oup[axis]) std::swap(lo, up);
        const int o0[3] = {gcm::kCornerX[lo], gcm::kCornerY[lo], gcm::kCornerZ[lo]};
        const int o1[3] = {gcm::kCornerX[up], gcm::kCornerY[up], gcm::kCornerZ[up]};
        const uint64_t plo = pidx(gp[0] + o0[0], gp[1] + o0[1], gp[2] + o0[2], nx, ny);
        const uint64_t pup = pidx(gp[0] + o1[0], gp[1] + o1[1], gp[2] + o1[2], nx, ny);
        const float t1 = acc[plo].t[axis];
        float t = t1;
        if (g) {
          const float f0 = g[plo], f1 = g[pup];
          float t2 = 0.0f;
          if (((f1 >= iso) && (f0 <= iso)) || ((f0 >= iso) && (f1 <= iso))) t2 = (iso - f0) / (f1 - f0);
          t = 0.0f;
          if ((t1 > 0) && (t2 > 0)) t = (float)((double)(t1 + t2) * 0.5);
          else if ((t1 > 0) && (t2 == 0)) t = t1;
          else if ((t2 > 0) && (t1 == 0)) t = t2;
        }
        for (int a = 0; a < 3; ++a) {
          const float d = (float)gp[a] - gc[a];
          vv[m][a] = lerp_axis(d, vs[a], o0[a], o1[a], t, A);
        }
      }
      float n[3];
      normal_of(vv[0], vv[2], vv[1], A.cross, n);
      const uint64_t idx = scan[v] + j;
      if (idx + 3 > capacity) continue;
      for (int m = 0; m < 3; ++m) {
        float* P = pos + 4 * (idx + m);
        float* N = norm + 4 * (idx + m);
        P[0] = vv[m][0]; P[1] = vv[m][1]; P[2] = vv[m][2]; P[3] = 1.0f;
        N[0] = n[0]; N[1] = n[1]; N[2] = n[2]; N[3] = 0.5f;
      }
    }
  }
  (void)nz;
  return total;
}

// The lattice previews of classifyVoxel and generateTriangles_lattice_kernel
// (src/MarchingCubes_kernel.cu:869-1052, 1865-2200) with `fixed` (mode 2: the
// primitive field f with the open lattice band iso1 < L < iso2; classic edge
// direction; vertexInterp_new :1728-1790) or `dynamic` (mode 3: the
// accumulated sign with the band, its difference keeping L < iso1 or L > iso2;
// edges from the lower corner; vertexInterp_primitive_one :1676-1726) set;
// normals calcNormal(v0, v2, v1) with w = 0.5.
static float preview_t_fixed(float iso, float i1, float i2, float f0, float f1, float f2, float f3) {
  float t1 = 0.0f, t2 = 0.0f, t3 = 0.0f;
  if (((f0 < iso) && (f1 >= iso)) || ((f1 < iso) && (f0 >= iso))) t1 = (iso - f0) / (f1 - f0);
  if (((f2 < i1) && (f3 >= i1)) || ((f3 < i1) && (f2 >= i1))) t2 = (i1 - f2) / (f3 - f2);
  if (((f2 < i2) && (f3 >= i2)) || ((f3 < i2) && (f2 >= i2))) t3 = (i2 - f2) / (f3 - f2);
  if ((t1 > 0.0f) && (t2 > 0.0f) && (t3 == 0.0f)) return (float)((double)(t1 + t2) * 0.5);
  if ((t1 > 0.0f) && (t3 > 0.0f) && (t2 == 0.0f)) return (float)((double)(t1 + t3) * 0.5);
  if ((t1 > 0.0f) && (t2 == 0.0f) && (t3 == 0.0f)) return t1;
  if ((t2 > 0.0f) && (t1 == 0.0f) && (t3 == 0.0f)) return t2;
  if ((t3 > 0.0f) && (t1 == 0.0f) && (t2 == 0.0f)) return t3;
  return 0.0f;
}

static float preview_t_dynamic(float i1, float i2, float f0, float f1, float t1) {
  float t2 = 0.0f, t3 = 0.0f, t = 0.0f;
  if (((f1 >= i1) && (f0 <= i1)) || ((f0 >= i1) && (f1 <= i1))) t2 = (i1 - f0) / (f1 - f0);
  if ((t1 > 0) && (t2 > 0)) t = (float)((double)(t1 + t2) * 0.5);
  else if ((t1 > 0) && (t2 == 0)) t = t1;
  else if ((t2 > 0) && (t1 == 0)) t = t2;
  if (((f1 >= i2) && (f0 <= i2)) || ((f0 >= i2) && (f1 <= i2))) t3 = (i2 - f0) / (f1 - f0);
  if ((t1 > 0) && (t3 > 0)) t = (float)((double)(t1 + t3) * 0.5);
  else if ((t1 > 0) && (t3 == 0)) t = t1;
  else if ((t3 > 0) && (t1 == 0)) t = t3;
  return t;
}

uint64_t orc_mesh_lattice_preview(const orc_csg_point* acc, const float* f, const float* L, uint32_t mode,
                                  uint32_t op, uint32_t nx, uint32_t ny, uint32_t nz, const float* vs,
                                  const float* gc, float iso, float iso1, float iso2, float* pos, float* norm,
                                  uint64_t capacity, uint64_t* active_out) {
  const bool fixed = mode == 2;
  const uint64_t nvox = (uint64_t)(nx - 1) * (ny - 1) * (nz - 1);
  auto inside = [&](uint64_t i) {
    const bool band = (L[i] > iso1) && (L[i] < iso2);
    if (fixed) {
      if (op == 1) return (f[i] >= iso) && band;
      if (op == 2) return (f[i] < iso) && band;
      return (f[i] < iso) || band;
    }
    const bool a = (float)acc[i].val < iso;
    if (op == 1) return a && ((L[i] < iso1) || (L[i] > iso2));
    if (op == 2) return a && band;
    return a || band;
  };
  auto cube = [&](uint32_t x, uint32_t y, uint32_t z) {
    unsigned ci = 0;
    for (int k = 0; k < 8; ++k)
      ci |= (unsigned)inside(pidx(x + gcm::kCornerX[k], y + gcm::kCornerY[k], z + gcm::kCornerZ[k], nx, ny)) << k;
    return ci;
  };
  std::vector<uint64_t> scan(nvox);
  uint64_t total = 0, active = 0;
  for (uint64_t v = 0; v < nvox; ++v) {
    uint32_t x, y, z;
    voxel_pos(v, nx, ny, x, y, z);
    const unsigned n = kNumVerts(cube(x, y, z));
    scan[v] = total;
    total += n;
    active += n > 0;
  }
  if (active_out) *active_out = active;
  const Arith A = decode(orc_default_arith());
  for (uint64_t v = 0; v < nvox; ++v) {
    uint32_t gp[3];
    voxel_pos(v, nx, ny, gp[0], gp[1], gp[2]);
    const unsigned ci = cube(gp[0], gp[1], gp[2]);
    const uint64_t row = gcm::kTriRows[ci];
    const unsigned nv = kNumVerts(ci);
    for (unsigned j = 0; j < nv; j += 3) {
      float vv[3][3];
      for (int m = 0; m < 3; ++m) {
        const int e = (int)gcm::tri_edge(row, j + m);
        int lo = gcm::kEdgeA[e], up = gcm::kEdgeB[e];
        int axis = 0;
        {
          const int olo[3] = {gcm::kCornerX[lo], gcm::kCornerY[lo], gcm::kCornerZ[lo]};
          const int oup[3] = {gcm::kCornerX[up], gcm::kCornerY[up], gcm::kCornerZ[up]};
          for (int a = 0; a < 3; ++a)
            if (olo[a] != oup[a]) axis = a;
          if (!fixed && olo[axis] > oup[axis]) std::swap(lo, up);  // dynamic: from the lower corner
        }
        const int o0[3] = {gcm::kCornerX[lo], gcm::kCornerY[lo], gcm::kCornerZ[lo]};
        const int o1[3] = {gcm::kCornerX[up], gcm::kCornerY[up], gcm::kCornerZ[up]};
        const uint64_t p0 = pidx(gp[0] + o0[0], gp[1] + o0[1], gp[2] + o0[2], nx, ny);
        const uint64_t p1 = pidx(gp[0] + o1[0], gp[1] + o1[1], gp[2] + o1[2], nx, ny);
        const float t = fixed ? preview_t_fixed(iso, iso1, iso2, f[p0], f[p1], L[p0], L[p1])
                              : preview_t_dynamic(iso1, iso2, L[p0], L[p1], acc[p0].t[axis]);
        for (int a = 0; a < 3; ++a) {
          const float d = (float)gp[a] - gc[a];
          vv[m][a] = lerp_axis(d, vs[a], o0[a], o1[a], t, A);
        }
      }
      float n[3];
      normal_of(vv[0], vv[2], vv[1], A.cross, n);
      const uint64_t idx = scan[v] + j;
      if (idx + 3 > capacity) continue;
      for (int m = 0; m < 3; ++m) {
        float* P = pos + 4 * (idx + m);
        float* N = norm + 4 * (idx + m);
        P[0] = vv[m][0]; P[1] = vv[m][1]; P[2] = vv[m][2]; P[3] = 1.0f;
        N[0] = n[0]; N[1] = n[1]; N[2] = n[2]; N[3] = 0.5f;
      }
    }
  }
  return total;
}

// ---- spatially variant lattices ---------------------------------------------------

// Coefficient m's frequencies: k outer, j, i inner over [-range, range]
// (src/main.cu:3615-3690).
static void svl_freq(uint32_t m, int range, int& i, int& j, int& k) {
  const int w = 2 * range + 1;
  i = (int)(m % w) - range;
  j = (int)((m / w) % w) - range;
  k = (int)(m / (w * w)) - range;
}

// Fourier coefficients of the sampled unit cell in double
// (c = (1/N) sum f e^{-2 pi i (ix/Nx + jy/Ny + kz/Nz)}, the R2C cuFFT scaled by
// 1/N and completed by symmetry in the reference, src/main.cu:3581-3690).
void orc_svl_dft(const float* f, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t range, float* out) {
  const uint32_t w = 2 * range + 1, nc = w * w * w;
  const double two_pi = 6.283185307179586476925286766559;
  for (uint32_t m = 0; m < nc; ++m) {
    int i, j, k;
    svl_freq(m, (int)range, i, j, k);
    double ar = 0, ai = 0;
    for (uint32_t z = 0; z < nz; ++z)
      for (uint32_t y = 0; y < ny; ++y)
        for (uint32_t x = 0; x < nx; ++x) {
          const double turns = (double)(((int64_t)i * x) % (int64_t)nx) / nx +
                               (double)(((int64_t)j * y) % (int64_t)ny) / ny +
                               (double)(((int64_t)k * z) % (int64_t)nz) / nz;
          const double v = f[x + (uint64_t)nx * (y + (uint64_t)ny * z)];
          ar += v * std::cos(-two_pi * turns);
          ai += v * std::sin(-two_pi * turns);
        }
    const double N = (double)nx * ny * nz;
    out[2 * m] = (float)(ar / N);
    out[2 * m + 1] = (float)(ai / N);
  }
}

namespace {
struct SvlSt {
  float a1, a2;
  int n1, n2;
};
SvlSt svl_stencil(int x, int n) {
  if (x == 0) return {-1.0f, -0.5f, x, x + 1};
  if (x == 1) return {1.0f, -0.5f, x - 1, x + 1};
  if (x == n - 2) return {0.5f, -1.0f, x - 1, x + 1};
  if (x == n - 1) return {0.5f, 1.0f, x - 1, x};
  return {0.5f, -0.5f, x - 1, x + 1};
}
inline float svl_k(float per, float v) { return (float)((2.0 * 3.14159265358979323846 / (double)per) * (double)v); }
}  // namespace

// finding_phi_kernel (src/lattice_files/Gratings.cu:100-417) for coefficient m:
// the stencil weights by boundary, the grating rotation by kind, the periods by
// period type; (2 pi / per) * (...) in double; i c - j s and i s + j c with the
// first product fused (nvcc's contraction in the reference build).
void orc_svl_rhs(const orc_svl* p, const float* period, uint32_t m, float* out) {
  const int X = (int)p->nx, Y = (int)p->ny, Z = (int)p->nz;
  int qi, qj, qk;
  svl_freq(m, (int)p->range, qi, qj, qk);
  const float fi = (float)qi, fj = (float)qj;
  for (int tx = 0; tx < X * Y * Z; ++tx) {
    const int x = tx % X, y = (tx % (X * Y)) / X, z = tx / (X * Y);
    const SvlSt sx = svl_stencil(x, X), sy = svl_stencil(y, Y), sz = svl_stencil(z, Z);
    float t1 = 0, t2 = 0, t3 = 0, t4 = 0, t5 = 0, t6 = 0, t7 = 0, t8 = 0;
    if (p->kind == 'r' || p->kind == 'b') {
      const float mx = p->kind == 'r' ? (float)(X + 1) / 2.0f : 0.0f, my = p->kind == 'r' ? (float)(Y + 1) / 2.0f : 0.0f;
      const float yy = ((float)(y + 1) - my) * p->dx;
      t1 = std::atan2(yy, ((float)(sx.n1 + 1) - mx) * p->dx);
      t2 = std::atan2(yy, ((float)(sx.n2 + 1) - mx) * p->dx);
      const float xx = ((float)(x + 1) - mx) * p->dx;
      t3 = std::atan2(((float)(sy.n1 + 1) - my) * p->dx, xx);
      t4 = std::atan2(((float)(sy.n2 + 1) - my) * p->dx, xx);
    } else if (p->kind == 's') {
      auto wave = [&](float u) { return p->lcon * std::sin((float)(6.28 * (double)p->lcon_1 * (double)u)); };
      t1 = wave((float)(sx.n1 + 1) * p->dx);
      t5 = wave((float)(sz.n1 + 1) * p->dz);
      t2 = wave((float)(sx.n2 + 1) * p->dx);
      t6 = wave((float)(sz.n2 + 1) * p->dz);
      t3 = wave((float)(x + 1) * p->dx);
      t7 = wave((float)(z + 1) * p->dz);
      t4 = t3;
      t8 = t7;
    }
    float p1, p2, p3, p4, p5, p6;
    if (p->period_type == 1) {
      p1 = p2 = p->period_x; p3 = p4 = p->period_y; p5 = p6 = p->period_z;
    } else if (p->period_type == 2) {
      p1 = period[sx.n1 + y * X + z * X * Y]; p2 = period[sx.n2 + y * X + z * X * Y];
      p3 = period[x + sy.n1 * X + z * X * Y]; p4 = period[x + sy.n2 * X + z * X * Y];
      p5 = period[x + y * X + sz.n1 * X * Y]; p6 = period[x + y * X + sz.n2 * X * Y];
    } else {
      p1 = p2 = p3 = p4 = p5 = p6 = p->period;
    }
    auto ra = [&](float th) { return std::fma(fi, std::cos(th), -(fj * std::sin(th))); };
    auto rb = [&](float th) { return std::fma(fi, std::sin(th), fj * std::cos(th)); };
    const float kx1 = svl_k(p1, ra(t1)), kx2 = svl_k(p2, ra(t2));
    const float ky1 = svl_k(p3, rb(t3)), ky2 = svl_k(p4, rb(t4));
    const float kz1 = (float)((2.0 * 3.14159265358979323846 / (double)p5) * (double)qk);
    const float kz2 = (float)((2.0 * 3.14159265358979323846 / (double)p6) * (double)qk);
    float phii = ((sx.a1 * kx1 + sx.a2 * kx2) + (sy.a1 * ky1 + sy.a2 * ky2)) + (sz.a1 * kz1 + sz.a2 * kz2);
    if (p->kind == 's' && p->sinewave_z) {
      const float fk = (float)qk;
      const float kz1b = svl_k(p5, std::fma(fj, std::sin(t5), fk * std::cos(t5)));
      const float kz2b = svl_k(p6, std::fma(fj, std::sin(t6), fk * std::cos(t6)));
      const float ky1b = svl_k(p3, std::fma(fj, std::cos(t7), -(fk * std::sin(t7))));
      const float ky2b = svl_k(p4, std::fma(fj, std::cos(t8), -(fk * std::sin(t8))));
      const float kx1b = (float)((2.0 * 3.14159265358979323846 / (double)p1) * (double)qi);
      const float kx2b = (float)((2.0 * 3.14159265358979323846 / (double)p2) * (double)qi);
      phii += ((sx.a1 * kx1b + sx.a2 * kx2b) + (sy.a1 * ky1b + sy.a2 * ky2b)) + (sz.a1 * kz1b + sz.a2 * kz2b);
    }
    out[tx] = phii;
  }
}

namespace {
// GPUMatvec_lattice_kernel (Gratings.cu:420-597)
void svl_axis(const float* dv, int c, int n, long st, float& w, float& t2, float& t3) {
  if (c == 0) { w = 1.25f; t2 = -dv[st]; t3 = -0.25f * dv[2 * st]; }
  else if (c == 1) { w = 1.25f; t2 = -dv[-st]; t3 = -0.25f * dv[2 * st]; }
  else if (c == n - 2) { w = 1.25f; t2 = -0.25f * dv[-2 * st]; t3 = -dv[st]; }
  else if (c == n - 1) { w = 1.25f; t2 = -0.25f * dv[-2 * st]; t3 = -dv[-st]; }
  else { w = 0.5f; t2 = -0.25f * dv[-2 * st]; t3 = -0.25f * dv[2 * st]; }
}
void svl_matvec(const float* d, float* q, int X, int Y, int Z) {
  for (int tx = 0; tx < X * Y * Z; ++tx) {
    const int x = tx % X, y = (tx % (X * Y)) / X, z = tx / (X * Y);
    float wx, x2, x3, wy, y2, y3, wz, z2, z3;
    svl_axis(d + tx, x, X, 1, wx, x2, x3);
    svl_axis(d + tx, y, Y, X, wy, y2, y3);
    svl_axis(d + tx, z, Z, (long)X * Y, wz, z2, z3);
    float a = std::fma((wx + wy) + wz, d[tx], x2);
    a = ((((a + x3) + y2) + y3) + z2) + z3;
    q[tx] = a;
  }
}
// GPUScalar_lattice_kernel + Reduction_lattice (Gratings.cu:22-75, 600-651):
// 1024-element blocks summed as a tree, then thread t of one 1024-thread block
// adds partials t, t + 1024, ... in sequence and the block sums as a tree.
float svl_tree(float* cc) {
  for (int s = 512; s > 0; s /= 2)
    for (int t = 0; t < s; ++t) cc[t] = cc[t] + cc[t + s];
  return cc[0];
}
float svl_dot(const float* a, const float* b, long n) {
  const long nb = (n + 1023) / 1024;
  std::vector<float> part(nb);
  float cc[1024];
  for (long blk = 0; blk < nb; ++blk) {
    for (int t = 0; t < 1024; ++t) {
      const long i = blk * 1024 + t;
      cc[t] = i < n ? a[i] * b[i] : 0.0f;
    }
    part[blk] = svl_tree(cc);
  }
  for (int t = 0; t < 1024; ++t) {
    float c = 0.0f;
    for (long k = 0; k * 1024 + t < nb; ++k) c += part[k * 1024 + t];
    cc[t] = c;
  }
  return svl_tree(cc);
}
// VecSMultAddKernel_lattice: v = a1 * v + a2 * w, the first product fused
void svl_axpby(float* v, float a1, const float* w, float a2, long n) {
  for (long i = 0; i < n; ++i) v[i] = std::fma(a1, v[i], a2 * w[i]);
}
}  // namespace

// Gratings::GPUCG_lattice (Gratings.cu:875-974) from x = 0: d = r = rhs,
// delta = r . d, steps while count < max_iter and delta > end_res^2.
uint32_t orc_svl_cg(const orc_svl* p, const float* rhs, float* x) {
  const int X = (int)p->nx, Y = (int)p->ny, Z = (int)p->nz;
  const long n = (long)X * Y * Z;
  std::vector<float> d(rhs, rhs + n), r(rhs, rhs + n), q(n, 0.0f);
  std::fill(x, x + n, 0.0f);
  float delta_new = svl_dot(r.data(), d.data(), n);
  const float term = p->end_res * p->end_res;
  uint32_t it = 1;
  while (it < p->max_iter && delta_new > term) {
    svl_matvec(d.data(), q.data(), X, Y, Z);
    const float dq = svl_dot(d.data(), q.data(), n);
    const float alpha = delta_new / dq;
    svl_axpby(x, 1.0f, d.data(), alpha, n);
    svl_axpby(r.data(), 1.0f, q.data(), (float)(-1.0 * (double)alpha), n);
    const float delta_old = delta_new;
    delta_new = svl_dot(r.data(), r.data(), n);
    const float beta = delta_new / delta_old;
    svl_axpby(d.data(), beta, r.data(), 1.0f, n);
    ++it;
  }
  return it;
}

// grating_kernel + svl_kernel (Gratings.cu:653-752) for m = 0 .. n_coeff-1: the
// phase sampled at (u/2 + 1/2, ...) of the coarse grid as a clamped linear
// texture (weights 0 or 1/2 per axis, x then y then z), exp(i phi), and
// svl += cos(phi) c.x - sin(phi) c.y, the first product fused.
void orc_svl_accumulate(const orc_svl* p, const float* phases, const float* coef, float* svl) {
  const int X = (int)p->nx, Y = (int)p->ny, Z = (int)p->nz;
  const long P = (long)X * Y * Z;
  const int FX = 2 * X, FY = 2 * Y, FZ = 2 * Z;
  for (int w = 0; w < FZ; ++w)
    for (int v = 0; v < FY; ++v)
      for (int u = 0; u < FX; ++u) {
        const int i0 = u >> 1, j0 = v >> 1, k0 = w >> 1;
        const int i1 = std::min(i0 + (u & 1), X - 1), j1 = std::min(j0 + (v & 1), Y - 1),
                  k1 = std::min(k0 + (w & 1), Z - 1);
        const float fx = (u & 1) ? 0.5f : 0.0f, fy = (v & 1) ? 0.5f : 0.0f, fz = (w & 1) ? 0.5f : 0.0f;
        float& acc = svl[u + (long)FX * (v + (long)FY * w)];
        for (uint32_t m = 0; m < p->n_coeff; ++m) {
          const float* xm = phases + m * P;
          auto at = [&](int i, int j, int k) { return xm[i + (long)X * (j + (long)Y * k)]; };
          auto lx = [&](int j, int k) { return std::fma(fx, at(i1, j, k) - at(i0, j, k), at(i0, j, k)); };
          const float c00 = lx(j0, k0), c10 = lx(j1, k0), c01 = lx(j0, k1), c11 = lx(j1, k1);
          const float c0 = std::fma(fy, c10 - c00, c00), c1 = std::fma(fy, c11 - c01, c01);
          const float ph = std::fma(fz, c1 - c0, c0);
          acc = acc + std::fma(std::cos(ph), coef[2 * m], -(std::sin(ph) * coef[2 * m + 1]));
        }
      }
}

// create_lattice_kernel (src/lattice_files/Fft_lattice.cu:11-93): unit cell on
// [-1, 1]^3 with the literal 3.14; the coordinate is formed in double and
// rounded to float, and the products with 3.14 are double, rounded to float at
// the call of cosf/sinf.
void orc_unit_cell(uint32_t type, uint32_t nx, uint32_t ny, uint32_t nz, float* out) {
  for (uint32_t z = 0; z < nz; ++z)
    for (uint32_t y = 0; y < ny; ++y)
      for (uint32_t x = 0; x < nx; ++x) {
        const float xx = (float)((((x * 1.0) / (nx - 1)) - 0.5) / 0.5);
        const float yy = (float)((((y * 1.0) / (ny - 1)) - 0.5) / 0.5);
        const float zz = (float)((((z * 1.0) / (nz - 1)) - 0.5) / 0.5);
        float aa = 0.0f;
        auto C = [](double v) { return cosf((float)v); };
        auto S = [](double v) { return sinf((float)v); };
        switch (type) {
          case 0: aa = C(3.14 * xx) * S(3.14 * yy) + C(3.14 * yy) * S(3.14 * zz) + C(3.14 * zz) * S(3.14 * xx); break;
          case 1: aa = C(3.14 * xx) + C(3.14 * yy) + C(3.14 * zz); break;
          case 2:
            aa = 4 * (cosf(xx) * cosf(yy) * cosf(zz)) -
                 (cosf(2 * xx) * cosf(2 * yy) + cosf(2 * yy) * cosf(2 * zz) + cosf(2 * zz) * cosf(2 * xx));
            break;
          case 3:
            aa = 2 * (C(3.14 * xx) * C(3.14 * yy) + C(3.14 * yy) * C(3.14 * zz) + C(3.14 * zz) * C(3.14 * xx)) -
                 (C(2 * 3.14 * xx) + C(2 * 3.14 * yy) + C(2 * 3.14 * zz));
            break;
          case 4:
            aa = (float)std::min(std::min((double)(powf(xx, 2)) + std::pow((double)yy, 2),
                                          std::pow((double)yy, 2) + std::pow((double)zz, 2)),
                                 std::pow((double)zz, 2) + std::pow((double)xx, 2));
            break;
          case 5:
            aa = (float)(std::cos(3.14 * xx) * C(3.14 * yy) * C(3.14 * zz) -
                         (double)(S(3.14 * xx) * S(3.14 * yy) * S(3.14 * zz)));
            break;
          default: aa = 0.0f;
        }
        out[pidx(x, y, z, nx, ny)] = aa;
      }
}

// One primitive on an Nx*Ny*Nz grid with the reference's centred coordinates
// x = (i - (N-1)/2) * dx (src/Modelling.cu:259-261 and the other kernels).
void orc_primitive(uint32_t kind, int nx, int ny, int nz, float dx, float dy, float dz, const float* center,
                   const float* v3, const float* p, uint32_t flag, float* out) {
  const float mx = (float)((nx - 1) / 2.0), my = (float)((ny - 1) / 2.0), mz = (float)((nz - 1) / 2.0);
  const float sp[3] = {dx, dy, dz};
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) {
        const float t[3] = {x - mx, y - my, z - mz};
        out[pidx(x, y, z, nx, ny)] = primitive_f32(kind, flag, center, v3, p, t, sp);
      }
}

void orc_lattice_field(const orc_lattice* L, uint32_t nx, uint32_t ny, uint32_t nz, float* out, int threads) {
  lattice_field_impl<false>(L, nx, ny, nz, out, threads);
}
void orc_lattice_field64(const orc_lattice* L, uint32_t nx, uint32_t ny, uint32_t nz, double* out, int threads) {
  lattice_field_impl<true>(L, nx, ny, nz, out, threads);
}
void orc_lattice_field_slab(const orc_lattice* L, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t z0,
                            uint32_t nplanes, float* out, int threads) {
  lattice_field_impl<false>(L, nx, ny, nz, out, threads, z0, nplanes);
}
void orc_lattice_field64_slab(const orc_lattice* L, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t z0,
                            uint32_t nplanes, double* out, int threads) {
  lattice_field_impl<true>(L, nx, ny, nz, out, threads, z0, nplanes);
}

void orc_csg_field(const orc_prim* prims, uint32_t n, const float* origin, const float* spacing, uint32_t nx,
                   uint32_t ny, uint32_t nz, float* out, int threads) {
  csg_impl<float>(prims, n, origin, spacing, nx, ny, nz, out, threads);
}
void orc_csg_field64(const orc_prim* prims, uint32_t n, const float* origin, const float* spacing, uint32_t nx,
                     uint32_t ny, uint32_t nz, double* out, int threads) {
  csg_impl<double>(prims, n, origin, spacing, nx, ny, nz, out, threads);
}

// GPU_buffer_normalise_four (src/lattice_files/Gratings.cu:1579-1617): the
// reference's final min/max reduction starts from {0, 0}
// (Min_reduction_lattice, :1439-1495), so the range always includes 0; then
// device_bufferfour (:1089-1134) maps k = (v - min) / (max - min), labels the
// band lo <= k <= hi with 1, and forces boundary samples to k = 0, label 0.
// set_period_kernel (src/lattice_files/Gratings.cu:818-860): sqrt((u+1)^2 +
// (v+1)^2) of the coordinates across the axis, x = (i - mean) * d; the
// reference build fuses (i - mean) * d + 1.  Squares here are correctly
// rounded (the reference's powf(v, 2) can differ in the last bit).
void orc_svl_period_field(uint32_t nx, uint32_t ny, uint32_t nz, const float* d, const float* mean, char axis,
                          float* out) {
  for (uint32_t zz = 0; zz < nz; ++zz)
    for (uint32_t yy = 0; yy < ny; ++yy)
      for (uint32_t xx = 0; xx < nx; ++xx) {
        const float x1 = std::fma((float)(int)xx - mean[0], d[0], 1.0f);
        const float y1 = std::fma((float)(int)yy - mean[1], d[1], 1.0f);
        const float z1 = std::fma((float)(int)zz - mean[2], d[2], 1.0f);
        float s;
        if (axis == 'z') s = x1 * x1 + y1 * y1;
        else if (axis == 'y') s = x1 * x1 + z1 * z1;
        else s = z1 * z1 + y1 * y1;
        out[pidx(xx, yy, zz, nx, ny)] = std::sqrt(s);
      }
}

// GPU_buffer_normalise_three (src/lattice_files/Gratings.cu:1539-1572) with
// device_bufferthree (:1071-1087): min/max starting from {0,0}, then
// a1 + b1 * (v - min) / (max - min), the reference build fusing a1 + b1 * k.
void orc_normalise_range(const float* in, float* out, uint64_t n, float a1, float b1, float* minmax) {
  float lo = 0.0f, hi = 0.0f;
  for (uint64_t i = 0; i < n; ++i) {
    lo = std::min(lo, in[i]);
    hi = std::max(hi, in[i]);
  }
  for (uint64_t i = 0; i < n; ++i) out[i] = std::fma(b1, (in[i] - lo) / (hi - lo), a1);
  if (minmax) {
    minmax[0] = lo;
    minmax[1] = hi;
  }
}

// primitive_field_kernel (src/lattice_files/Gratings.cu:1695-1725).
void orc_lattice_mask(const orc_csg_point* acc, const float* prim, float* lat, uint64_t n, int fixed, int dynamic) {
  for (uint64_t i = 0; i < n; ++i) {
    if (fixed) {
      if ((float)acc[i].val > -1.0f) lat[i] = FLT_MAX;
    } else if (dynamic) {
      if (prim[i] >= 0.0f) lat[i] = FLT_MAX;
    }
  }
}

void orc_normalise_band(const float* field, int nx, int ny, int nz, float lo, float hi, float* label, float* nf,
                        float* minmax) {
  const uint64_t total = (uint64_t)nx * ny * nz;
  float a = 0.0f, b = 0.0f;
  for (uint64_t i = 0; i < total; ++i) {
    a = std::min(a, field[i]);
    b = std::max(b, field[i]);
  }
  if (minmax) { minmax[0] = a; minmax[1] = b; }
  for (uint64_t i = 0; i < total; ++i) {
    const int xx = (int)(i % nx), yy = (int)((i / nx) % ny), zz = (int)(i / ((uint64_t)nx * ny));
    float k = (field[i] - a) / (b - a), m;
    if (xx == 0 || xx == nx - 1 || yy == 0 || yy == ny - 1 || zz == 0 || zz == nz - 1) {
      m = 0.0f;
      k = 0.0f;
    } else {
      m = (k >= lo && k <= hi) ? 1.0f : 0.0f;
    }
    label[i] = m;
    nf[i] = k;
  }
}

// File_output::file_write_obj (src/File_output.cu:5-81): positions truncated to a
// 0.001 grid (int(x*1000)*0.001, rounded back to float), welded on first
// occurrence with 1-based indices, faces with a repeated index dropped,
// identical ordered faces written once, winding written as (a, c, b).
int orc_write_obj(const float* pos, uint64_t nverts, const char* path, uint64_t* nv_out, uint64_t* nf_out) {
  std::ofstream f(path, std::ios::out);
  if (!f) return 1;
  f << "##Sample latttice new Obj \n";
  f << "o Solid \n";
  std::map<std::vector<float>, int> vmap;
  std::vector<uint32_t> faces;
  faces.reserve(nverts);
  int index = 0;
  for (uint64_t i = 0; i < nverts; ++i) {
    const float vx = (float)(int(pos[4 * i + 0] * 1000) * 0.001);
    const float vy = (float)(int(pos[4 * i + 1] * 1000) * 0.001);
    const float vz = (float)(int(pos[4 * i + 2] * 1000) * 0.001);
    std::vector<float> key = {vx, vy, vz};
    auto it = vmap.find(key);
    if (it == vmap.end()) {
      ++index;
      vmap.emplace(key, index);
      faces.push_back((uint32_t)index);
      f << "v " << vx << " " << vy << " " << vz << "\n";
    } else {
      faces.push_back((uint32_t)it->second);
    }
  }
  f << "\n";
  f << "\n";
  std::map<std::vector<uint32_t>, int> fmap;
  uint64_t nfaces = 0;
  for (uint64_t i = 0; i + 2 < faces.size(); i += 3) {
    const uint32_t a = faces[i], b = faces[i + 1], c = faces[i + 2];
    if (a != b && a != c && b != c) {
      std::vector<uint32_t> key = {a, b, c};
      if (fmap.count(key) == 0) {
        fmap[key] = 1;
        f << " f  " << a << " " << c << " " << b << "\n";
        ++nfaces;
      }
    }
  }
  if (nv_out) *nv_out = (uint64_t)index;
  if (nf_out) *nf_out = nfaces;
  return f.good() ? 0 : 2;
}

}  // extern "C"
