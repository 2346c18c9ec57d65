// CPU oracle for the field -> mesh path.  TEST INFRASTRUCTURE ONLY: the tests,
// the smoke check and bench.py's CPU-baseline leg call it to check and time
// against; the product never links, loads or falls back to it.
//
// Each function restates one piece of the reference (DESIGN4ADDITIVE/GPUCADforAM)
// and cites the file:line it follows.  Grid conventions are the reference's:
// nx*ny*nz FP32 samples with x fastest; voxel (x,y,z) spans samples x..x+1,
// y..y+1, z..z+1; voxels are numbered x fastest over (nx-1)(ny-1)(nz-1)
// (calcGridPos, src/MarchingCubes_kernel.cu:121-136).
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

// Floating-point contraction pattern of the vertex arithmetic (see oracle.cpp).
// bit 0     : corner at offset 1 computed as fma(d, vs, vs) instead of d*vs + vs
// bit 1     : edge delta fused with the corner product
// bits 2..3 : lerp form (0 unfused, 1 fma(t, B, a), 2 fma(d, vs, t*B))
// bits 4..5 : cross-product form (0 unfused, 1 fma(a, b, -(c*d)), 2 fma(-c, d, a*b))
uint32_t orc_default_arith(void);

// ---- marching cubes on a fed field -------------------------------------------------
void orc_mc_classify(const float* field, uint32_t nx, uint32_t ny, uint32_t nz, float iso,
                     uint32_t* voxel_verts, uint32_t* voxel_occupied, uint8_t* cube_index);
uint64_t orc_scan_exclusive_u32(const uint32_t* in, uint32_t* out, uint64_t n);
void orc_mc_compact(const uint32_t* occupied, const uint32_t* occupied_scan, uint64_t n,
                    uint32_t* compacted);
void orc_mc_generate(const float* field, uint32_t nx, uint32_t ny, uint32_t nz, const float* voxel_size,
                     const float* grid_center, float iso, const uint32_t* compacted, uint64_t active,
                     const uint32_t* verts_scan, uint64_t capacity_verts, float* pos, float* norm,
                     uint32_t arith);
void orc_mc_generate_band(const float* label, const float* norm_field, uint32_t nx, uint32_t ny, uint32_t nz,
                          const float* voxel_size, const float* grid_center, float iso, float band_lo,
                          float band_hi, const uint32_t* compacted, uint64_t active,
                          const uint32_t* verts_scan, uint64_t capacity_verts, float* pos, float* norm,
                          uint32_t arith);
// Whole pipeline (classify, scans, compact, generate), OpenMP-parallel.  Returns the
// vertex total; writes at most capacity_verts vertices.  band: label/norm_field mode.
uint64_t orc_mesh_field(const float* field, uint32_t nx, uint32_t ny, uint32_t nz, const float* voxel_size,
                        const float* grid_center, float iso, float* pos, float* norm, uint64_t capacity_verts,
                        uint64_t* active_out, int threads);

// ---- fields -----------------------------------------------------------------------
void orc_unit_cell(uint32_t type, uint32_t nx, uint32_t ny, uint32_t nz, float* out);
void orc_primitive(uint32_t kind, int nx, int ny, int nz, float dx, float dy, float dz, const float* center,
                   const float* v3, const float* p, uint32_t flag, float* out);

// Graded lattice, see oracle.cpp for the exact formulation.  The float forms
// restate the GPU's compensated arithmetic (pairs of floats through the reduced
// phase); the double forms are the accuracy reference.
typedef struct orc_lattice {
  uint32_t mode;  // 0 = trilinear parameters, 1 = trilinear blend of per-control-point fields
  uint32_t cx, cy, cz;
  const float* period;     // [cz*cy*cx], voxels
  const float* euler;      // [3][cz*cy*cx] radians, or NULL
  const float* thickness;  // [cz*cy*cx] or NULL
  const uint8_t* type;     // [cz*cy*cx]
  float origin[3];         // phase origin (voxel units), mode 0 only
} orc_lattice;
void orc_lattice_field(const orc_lattice* L, uint32_t nx, uint32_t ny, uint32_t nz, float* out, int threads);
void orc_lattice_field64(const orc_lattice* L, uint32_t nx, uint32_t ny, uint32_t nz, double* out, int threads);
// Planes z0 .. z0+nplanes-1 of the same nx*ny*nz field.
void orc_lattice_field_slab(const orc_lattice* L, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t z0,
                            uint32_t nplanes, float* out, int threads);
void orc_lattice_field64_slab(const orc_lattice* L, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t z0,
                              uint32_t nplanes, double* out, int threads);

// CSG scene of primitives: f = op_n(...op_1(op_0(+inf, g_0), g_1)..., g_n).
typedef struct orc_prim {
  uint32_t kind;  // see orc_primitive
  uint32_t op;    // 0 union (min), 1 subtract (max(f,-g)), 2 intersect (max)
  uint32_t flag;  // shell / disc selector
  uint32_t pad;
  float center[3];
  float v3[3];
  float p[6];
} orc_prim;
void orc_csg_field(const orc_prim* prims, uint32_t n, const float* origin, const float* spacing, uint32_t nx,
                   uint32_t ny, uint32_t nz, float* out, int threads);
void orc_csg_field64(const orc_prim* prims, uint32_t n, const float* origin, const float* spacing, uint32_t nx,
                     uint32_t ny, uint32_t nz, double* out, int threads);

// ---- band normalisation -------------------------------------------------------------
void orc_normalise_band(const float* field, int nx, int ny, int nz, float band_lo, float band_hi, float* label,
                        float* norm_field, float* minmax);

// SVL period field (set_period_kernel), min/max range map
// (GPU_buffer_normalise_three) and the lattice mask (primitive_field_kernel).
void orc_svl_period_field(uint32_t nx, uint32_t ny, uint32_t nz, const float* d, const float* mean, char axis,
                          float* out);
void orc_normalise_range(const float* in, float* out, uint64_t n, float a1, float b1, float* minmax);
struct orc_csg_point;
void orc_lattice_mask(const struct orc_csg_point* acc, const float* prim, float* lat, uint64_t n, int fixed,
                      int dynamic);

// ---- .obj -----------------------------------------------------------------------------
int orc_write_obj(const float* pos, uint64_t nverts, const char* path, uint64_t* nv_out, uint64_t* nf_out);

/* Retained primitive accumulation (grid_points, src/MarchingCubes_kernel.h:12-18)
 * and its meshes.  op: 0 union, 1 subtract, 2 intersect. */
typedef struct orc_csg_point {
  int32_t val;
  float t[3];
} orc_csg_point;
void orc_csg_retain(orc_csg_point* acc, const float* field, uint32_t nx, uint32_t ny, uint32_t nz, float iso,
                    uint32_t op);
/* The same fold with the open band iso1 < lattice < iso2 as the object. */
void orc_csg_retain_band(orc_csg_point* acc, const float* lattice, uint32_t nx, uint32_t ny, uint32_t nz, float iso,
                         float iso1, float iso2, uint32_t op);
/* field NULL: region mesh; else the accumulator combined with field by op.
 * Returns the vertex total; writes the triangles whose vertices fit. */
uint64_t orc_mesh_retained(const orc_csg_point* acc, const float* field, uint32_t op, uint32_t nx, uint32_t ny,
                           uint32_t nz, const float* voxel_size, const float* grid_center, float iso, float* pos,
                           float* norm, uint64_t capacity, uint64_t* active_out);
/* Lattice previews: mode 2 combines the primitive field with the open band
 * iso1 < lattice < iso2, mode 3 the accumulator with that band. */
uint64_t orc_mesh_lattice_preview(const orc_csg_point* acc, const float* field, const float* lattice, uint32_t mode,
                                  uint32_t op, uint32_t nx, uint32_t ny, uint32_t nz, const float* voxel_size,
                                  const float* grid_center, float iso, float iso1, float iso2, float* pos, float* norm,
                                  uint64_t capacity, uint64_t* active_out);

/* Spatially variant lattice (src/lattice_files/Gratings.cu:100-1050,
 * src/main.cu:3578-3711, 3904-4030). */
typedef struct orc_svl {
  uint32_t nx, ny, nz;
  float dx, dy, dz;
  uint32_t kind, period_type;
  float period, period_x, period_y, period_z, lcon, lcon_1;
  uint32_t sinewave_z, range, n_coeff, max_iter;
  float end_res;
} orc_svl;
void orc_svl_dft(const float* f, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t range, float* out);
void orc_svl_rhs(const orc_svl* p, const float* period, uint32_t m, float* out);
/* conjugate gradients from x = 0 on A x = rhs; returns the final step count */
uint32_t orc_svl_cg(const orc_svl* p, const float* rhs, float* x);
void orc_svl_accumulate(const orc_svl* p, const float* phases, const float* coef, float* svl);

#ifdef __cplusplus
}
#endif
