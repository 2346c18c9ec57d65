/*
 * gcm.h - C ABI of the GB300-native implicit-geometry meshing engine.
 *
 * Drop-in boundary for the field -> mesh path of DESIGN4ADDITIVE/GPUCADforAM.
 * The reference exposes that path as C++ classes (MarchingCubeCuda,
 * Isosurface, Modelling, Fft_lattice, Gratings, File_output); every entry
 * point below names the reference member it replaces (path:line inside the
 * reference project).
 *
 * Conventions shared by every call:
 *  - Grids hold nx*ny*nz FP32 samples, x fastest (index x + nx*(y + ny*z)).
 *    Voxel (x,y,z) spans samples x..x+1, y..y+1, z..z+1; voxels are numbered
 *    x fastest over (nx-1)*(ny-1)*(nz-1)  (calcGridPos,
 *    src/MarchingCubes_kernel.cu:121-136).
 *  - Meshes are unshared triangles: vertex i has position pos[4i..4i+3] =
 *    (x, y, z, 1) and normal norm[4i..4i+3] = (n, 0), triangle t = vertices
 *    3t..3t+2, in the reference's order (vertex index = exclusive scan of the
 *    per-voxel vertex counts in voxel order, then the triangle-table order).
 *  - Pointers named d_* are device pointers; h_* are host pointers.  The
 *    caller owns inputs and outputs.  Scratch is owned by the context.
 *  - `stream` is a cudaStream_t (NULL = the legacy default stream).  Calls
 *    that return host-side counts synchronise that stream; *_async calls do
 *    not and write their counts to device memory.
 *  - Every call returns a gcm_status; nothing exits or aborts.  On
 *    GCM_ERR_OUTPUT_OVERFLOW the true counts are still reported and only the
 *    triangles that fit were written.
 *  - A context is not thread-safe; use one context per host thread.
 */
#ifndef GCM_H_
#define GCM_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* The library is built with hidden visibility; everything declared here is
 * its exported interface. */
#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

#define GCM_ABI_VERSION 1

typedef enum gcm_status {
  GCM_OK = 0,
  GCM_ERR_INVALID_ARGUMENT = 1,
  GCM_ERR_OUTPUT_OVERFLOW = 2, /* capacity too small; counts are the true ones */
  GCM_ERR_DEVICE_TIMEOUT = 3,  /* a bounded device-side wait gave up */
  GCM_ERR_CUDA = 4,            /* a CUDA runtime call failed; see gcm_ctx_last_error */
  GCM_ERR_OUT_OF_MEMORY = 5,
  GCM_ERR_NOT_SUPPORTED = 6,
  GCM_ERR_IO = 7,
  GCM_ERR_REJECTED = 8,  /* server admission refused the request */
  GCM_ERR_CANCELLED = 9, /* server request cancelled before completion */
  GCM_ERR_BUSY = 10      /* server queue full */
} gcm_status;

typedef struct gcm_ctx gcm_ctx;
typedef void* gcm_stream; /* cudaStream_t */

/* Grid geometry.  Vertex positions are (gridPos - grid_center) * voxel_size,
 * as in generateTriangles_* (src/MarchingCubes_kernel.cu:3061-3064). */
typedef struct gcm_grid {
  uint32_t nx, ny, nz;
  float voxel_size[3];  /* reference: voxelSize  */
  float grid_center[3]; /* reference: gridcenter, in voxel units */
} gcm_grid;

/* Counts of one extraction (reference: *activeVoxels, *totalVerts,
 * src/Isosurface.cu:80,114). */
typedef struct gcm_counts {
  uint64_t active_voxels;
  uint64_t total_verts;
  uint32_t status; /* gcm_status of the device work (0 = ok) */
  uint32_t reserved;
} gcm_counts;

/* ---------------------------------------------------------------- context */

/* Creates a context on `device` (replaces the reference's global state:
 * texture objects src/MarchingCubes_kernel.cu:20-21 and the caller-side
 * scratch of src/main.cu:2141-2151). */
gcm_status gcm_ctx_create(int device, gcm_ctx** out);
gcm_status gcm_ctx_destroy(gcm_ctx* ctx);
const char* gcm_status_string(gcm_status s);
/* Text of the last error raised on this context ("" if none). */
const char* gcm_ctx_last_error(const gcm_ctx* ctx);
/* Grows the context's scratch so that meshing grids of up to max_points
 * samples allocates nothing afterwards (needed before stream capture). */
gcm_status gcm_ctx_reserve(gcm_ctx* ctx, uint64_t max_points);
/* Upper bound, in nanoseconds, on every device-side wait (decoupled
 * look-back).  Default 2e9.  A wait that runs out sets
 * GCM_ERR_DEVICE_TIMEOUT and the kernel returns. */
gcm_status gcm_ctx_set_wait_limit(gcm_ctx* ctx, uint64_t ns);
/* Extraction path of plain meshes (gcm_mesh_field, gcm_mesh_field_async,
 * gcm_mesh_lattice*, gcm_mesh_csg).  FUSED: one pass over tiles of whole
 * voxel rows with a decoupled look-back (best for dense surfaces, such as
 * graded lattices).  SPARSE: count the triangles of every 32-voxel window,
 * scan, and emit only the windows that hold triangles (best when the surface
 * touches a few percent of the voxels, such as primitive scenes).  AUTO
 * (default): SPARSE for gcm_mesh_csg, FUSED otherwise.  Every path writes the
 * same vertices in the same order.  No reference counterpart: the reference
 * runs classify, two thrust scans, compaction and generate
 * (src/Isosurface.cu:401-486). */
typedef enum gcm_mesh_path { GCM_MESH_PATH_AUTO = 0, GCM_MESH_PATH_FUSED = 1, GCM_MESH_PATH_SPARSE = 2 } gcm_mesh_path;
gcm_status gcm_ctx_set_mesh_path(gcm_ctx* ctx, gcm_mesh_path path);
/* Number of kernel launches this context has issued (for accounting). */
uint64_t gcm_ctx_launch_count(const gcm_ctx* ctx);
int gcm_abi_version(void);

/* ------------------------------------------------- marching cubes, fed field */

/* One fused pass over a caller-supplied FP32 field: classify, decoupled
 * look-back scan, and triangle emission.  Replaces
 * Isosurface::computeIsosurface_lattice / computeIsosurface_latticeone
 * (src/Isosurface.cu:401-572) in their plain form (cube index
 * classifyVoxel_new :3207-3249, interpolation vertexInterp4 :1619-1629,
 * normal calcNormal(v0,v1,v2) :1631-1637).  Host counts; syncs `stream`. */
gcm_status gcm_mesh_field(gcm_ctx* ctx, const float* d_field, const gcm_grid* grid, float iso, float* d_pos,
                          float* d_norm, uint64_t capacity_verts, gcm_counts* h_counts, gcm_stream stream);
/* Same, stream-ordered: counts land in d_counts (device), nothing syncs. */
gcm_status gcm_mesh_field_async(gcm_ctx* ctx, const float* d_field, const gcm_grid* grid, float iso, float* d_pos,
                                float* d_norm, uint64_t capacity_verts, gcm_counts* d_counts, gcm_stream stream);
/* Counting pass only (exact vertex total for admission / sizing). */
gcm_status gcm_count_field(gcm_ctx* ctx, const float* d_field, const gcm_grid* grid, float iso,
                           gcm_counts* h_counts, gcm_stream stream);

/* ---------------------------------- staged form (the reference's own steps) */

/* classifyVoxel_new (src/MarchingCubes_kernel.cu:3207-3249): per voxel vertex
 * count and occupancy flag; d_cube_index (optional) gets the 8-bit case. */
gcm_status gcm_mc_classify(gcm_ctx* ctx, const float* d_field, const gcm_grid* grid, float iso,
                           uint32_t* d_voxel_verts, uint32_t* d_voxel_occupied, uint8_t* d_cube_index,
                           gcm_stream stream);
/* ThrustScanWrapper_lattice (src/MarchingCubes_kernel.cu:3198-3203): exclusive
 * scan of n uint32 values (32-bit wrap-around, like thrust on uint), single
 * pass with decoupled look-back.  h_total (optional, syncs) gets the 64-bit sum. */
gcm_status gcm_scan_exclusive_u32(gcm_ctx* ctx, const uint32_t* d_in, uint32_t* d_out, uint64_t n,
                                  uint64_t* h_total, gcm_stream stream);
/* compactVoxels (src/MarchingCubes_kernel.cu:1594-1608). */
gcm_status gcm_mc_compact(gcm_ctx* ctx, const uint32_t* d_voxel_occupied, const uint32_t* d_occupied_scan, uint64_t n,
                          uint32_t* d_compacted, gcm_stream stream);
/* generateTriangles_lattice_kernel_3 (src/MarchingCubes_kernel.cu:3041-3170)
 * with the classify cube index. */
gcm_status gcm_mc_generate(gcm_ctx* ctx, const float* d_field, const gcm_grid* grid, float iso,
                           const uint32_t* d_compacted, uint64_t active_voxels, const uint32_t* d_verts_scan,
                           float* d_pos, float* d_norm, uint64_t capacity_verts, gcm_stream stream);

/* --------------------------------------------------------------- band mode */

/* GPU_buffer_normalise_four (src/lattice_files/Gratings.cu:1579-1617):
 * min/max (the range always includes 0, as the reference's reduction starts
 * from {0,0}), k = (v-min)/(max-min), label 1 where lo <= k <= hi, boundary
 * samples forced to k = 0, label 0.  h_minmax (optional, syncs) gets min,max. */
gcm_status gcm_normalise_band(gcm_ctx* ctx, const float* d_field, uint32_t nx, uint32_t ny, uint32_t nz, float band_lo,
                              float band_hi, float* d_label, float* d_norm_field, float* h_minmax, gcm_stream stream);
/* GPU_buffer_normalise_three (src/lattice_files/Gratings.cu:1539-1572,
 * device_bufferthree :1071-1087): min/max over the n values (the range always
 * includes 0, as the reference's reduction starts from {0,0}), then
 * v -> range_lo + range_span * (v - min) / (max - min).  d_in may equal d_out
 * (the reference maps its period field in place).  h_minmax (optional, syncs)
 * gets min, max. */
gcm_status gcm_normalise_range(gcm_ctx* ctx, const float* d_in, float* d_out, uint64_t n, float range_lo,
                               float range_span, float* h_minmax, gcm_stream stream);
/* Band extraction: cube index from the label field (< iso), vertices from the
 * normalised field at the band edges with the reference's 0.0005 endpoint
 * snapping.  Replaces computeIsosurface_lattice / _latticeone with
 * generateTriangles_lattice_kernel_new / _newone
 * (src/MarchingCubes_kernel.cu:3424-3817). */
gcm_status gcm_mesh_band(gcm_ctx* ctx, const float* d_label, const float* d_norm_field, const gcm_grid* grid, float iso,
                         float band_lo, float band_hi, float* d_pos, float* d_norm, uint64_t capacity_verts,
                         gcm_counts* h_counts, gcm_stream stream);
/* Same, stream-ordered: counts land in d_counts (device), nothing syncs. */
gcm_status gcm_mesh_band_async(gcm_ctx* ctx, const float* d_label, const float* d_norm_field, const gcm_grid* grid,
                               float iso, float band_lo, float band_hi, float* d_pos, float* d_norm,
                               uint64_t capacity_verts, gcm_counts* d_counts, gcm_stream stream);

/* ------------------------------------------------------------------ fields */

/* TPMS types: the reference's lattice_index_type values
 * (src/lattice_files/Fft_lattice.cu:59-85; names src/ImguiApp.cpp:2571). */
typedef enum gcm_tpms {
  GCM_TPMS_GYROID = 0,
  GCM_TPMS_SCHWARZ_P = 1,
  GCM_TPMS_FRD = 2,
  GCM_TPMS_IWP = 3,
  GCM_TPMS_CROSS_CUBE = 4, /* unit cell only */
  GCM_TPMS_SCHWARZ_D = 5   /* "diamond" */
} gcm_tpms;

/* create_lattice_kernel (src/lattice_files/Fft_lattice.cu:11-93): unit cell on
 * [-1,1]^3 (literal 3.14 as in the reference). */
gcm_status gcm_field_unit_cell(gcm_ctx* ctx, uint32_t type, uint32_t nx, uint32_t ny, uint32_t nz, float* d_out,
                               gcm_stream stream);

typedef enum gcm_grade_mode {
  /* period, Euler angles and thickness trilinear from the control grid, type
   * of the nearest control point, phase about `origin` */
  GCM_GRADE_PARAMS = 0,
  /* each control point anchors its own uniform lattice at its position; the
   * field is the trilinear blend of the 8 surrounding lattices */
  GCM_GRADE_BLEND = 1
} gcm_grade_mode;

/* Spatially graded TPMS lattice (the reference grades period, rotation and
 * thickness through Interpolations / Gratings: src/lattice_files/Gratings.cu:
 * 345-379 period, :260-341 rotation, :1089-1134 thickness band, trilinear
 * lookup src/Interpolations.cu:79-107).  Control arrays are device arrays of
 * cx*cy*cz values, x fastest; control point (i,j,k) sits at voxel position
 * (i*(nx-1)/(cx-1), ...).  Field = TPMS(R(euler) (p - origin) * 2pi/period)
 * - thickness, where R uses the Euler basis of src/Modelling.cu:401-407. */
typedef struct gcm_lattice {
  uint32_t mode; /* gcm_grade_mode */
  uint32_t cx, cy, cz;
  const float* d_period;    /* voxels */
  const float* d_euler;     /* [3][cx*cy*cz] radians (x, y, z), or NULL */
  const float* d_thickness; /* or NULL */
  const uint8_t* d_type;    /* gcm_tpms per control point (not CROSS_CUBE) */
  float origin[3];          /* GCM_GRADE_PARAMS phase origin (voxel units) */
} gcm_lattice;

gcm_status gcm_field_lattice(gcm_ctx* ctx, const gcm_lattice* lattice, uint32_t nx, uint32_t ny, uint32_t nz,
                             float* d_out, gcm_stream stream);
/* Field evaluation + marching cubes (iso usually 0). */
gcm_status gcm_mesh_lattice(gcm_ctx* ctx, const gcm_lattice* lattice, const gcm_grid* grid, float iso, float* d_pos,
                            float* d_norm, uint64_t capacity_verts, gcm_counts* h_counts, gcm_stream stream);
/* Same, stream-ordered: counts land in d_counts (device), nothing syncs, so
 * consecutive calls on one stream overlap with copies on other streams. */
gcm_status gcm_mesh_lattice_async(gcm_ctx* ctx, const gcm_lattice* lattice, const gcm_grid* grid, float iso,
                                  float* d_pos, float* d_norm, uint64_t capacity_verts, gcm_counts* d_counts,
                                  gcm_stream stream);

/* Primitive kinds (src/Modelling.cu): 0 sphere / sphere shell (flag) :314-361,
 * 1 capped cylinder / disc (flag) :244-302, 2 cuboid :375-421, 3 cuboid shell
 * :435-487, 4 torus :569-616, 5 cone :631-683, 6 cone frustum :698-750,
 * 7 pyramid frustum :501-557.  Parameters p[] in the reference's order:
 * sphere (radius, thickness); cylinder (radius, thickness_radial,
 * thickness_axial) with v3 = axis; cuboid (x_width, y_width, z_width) with
 * v3 = Euler angles; cuboid shell (+thickness); torus (R, r); cone
 * (base_radius, height); cone frustum (top_radius, bottom_radius, height);
 * pyramid frustum (x_base, x_top, y_height, z_base, z_top). */
typedef enum gcm_csg_op { GCM_CSG_UNION = 0, GCM_CSG_SUBTRACT = 1, GCM_CSG_INTERSECT = 2 } gcm_csg_op;
typedef struct gcm_primitive {
  uint32_t kind;
  uint32_t op;   /* gcm_csg_op applied to the running field */
  uint32_t flag; /* shell (sphere) / disc (cylinder) selector */
  uint32_t reserved;
  float center[3];
  float v3[3];
  float p[6];
} gcm_primitive;

/* Scene frame: sample i sits at (i - origin) * spacing (the reference uses
 * origin = (N-1)/2, spacing = dx; src/Modelling.cu:259-261). */
typedef struct gcm_frame {
  float origin[3];
  float spacing[3];
} gcm_frame;

/* Rounding of the primitive fields (the kernels of src/Modelling.cu:244-750).
 * DEFAULT follows the reference build's operation order and fused
 * multiply-adds with correctly rounded squares: within a few ulp of the
 * reference's fields (its powf(v, 2) differs from the rounded square in the
 * last bit for about 6% of floats).  REFERENCE squares with CUDA's powf as the
 * reference does and reproduces its fields bit for bit, at about 4x the cost
 * of the default on primitive-heavy scenes. */
typedef enum gcm_prim_arith { GCM_PRIM_ARITH_DEFAULT = 0, GCM_PRIM_ARITH_REFERENCE = 1 } gcm_prim_arith;
/* Selects the primitive arithmetic of this context's CSG calls
 * (gcm_field_csg, gcm_mesh_csg).  No reference counterpart: the reference has
 * only the powf form. */
gcm_status gcm_ctx_set_primitive_arith(gcm_ctx* ctx, gcm_prim_arith arith);

/* CSG field: f = op_n(... op_0(+inf, g_0) ..., g_n) with union = min,
 * subtract = max(f, -g), intersect = max(f, g).  d_prims is a device array. */
gcm_status gcm_field_csg(gcm_ctx* ctx, const gcm_primitive* d_prims, uint32_t n_prims, const gcm_frame* frame,
                         uint32_t nx, uint32_t ny, uint32_t nz, float* d_out, gcm_stream stream);
/* Field + extraction of a CSG scene in one call (the context keeps the field).
 * The field kernel records, per 32 x 8 x 8 sample tile, whether an enclosure
 * of the folded field lies wholly below or above iso; the windowed extraction
 * (the default for CSG, GCM_MESH_PATH_AUTO) then reads only the samples of
 * tiles that can hold the surface.  The same vertices as gcm_field_csg
 * followed by gcm_mesh_field. */
gcm_status gcm_mesh_csg(gcm_ctx* ctx, const gcm_primitive* d_prims, uint32_t n_prims, const gcm_frame* frame,
                        const gcm_grid* grid, float iso, float* d_pos, float* d_norm, uint64_t capacity_verts,
                        gcm_counts* h_counts, gcm_stream stream);
/* The same with the counts written to device memory, without a host
 * synchronisation. */
gcm_status gcm_mesh_csg_async(gcm_ctx* ctx, const gcm_primitive* d_prims, uint32_t n_prims, const gcm_frame* frame,
                              const gcm_grid* grid, float iso, float* d_pos, float* d_norm, uint64_t capacity_verts,
                              gcm_counts* d_counts, gcm_stream stream);

/* ------------------------------------------------- retained CSG accumulation */

/* The reference's interactive primitive editing keeps the model as a grid of
 * these (grid_points, src/MarchingCubes_kernel.h:12-18): per sample an inside
 * sign (-1 inside, 1 outside, 0 never touched) and the crossing fraction on
 * its +x, +y and +z edges, averaged over the primitives that crossed it.
 * A zeroed array is the empty model.  16 bytes per sample, x fastest. */
typedef struct gcm_csg_point {
  int32_t val;
  float t_x, t_y, t_z;
} gcm_csg_point;

/* Folds one primitive field into the accumulator with op
 * (Isosurface::copy_parameter -> classify_copy_Voxel static mode,
 * src/Isosurface.cu:16-27, src/MarchingCubes_kernel.cu:158-447).  The field
 * has the accumulator's nx*ny*nz samples; the reference folds at iso 0. */
gcm_status gcm_csg_retain(gcm_ctx* ctx, gcm_csg_point* d_acc, const float* d_field, uint32_t nx, uint32_t ny,
                          uint32_t nz, float iso, gcm_csg_op op, gcm_stream stream);
/* Folds a lattice band instead (classify_copy_Voxel with dynamic = true,
 * src/MarchingCubes_kernel.cu:158-447; its `fixed` flag is not read): the
 * object is band_lo < lattice < band_hi, each edge's fraction is where the
 * lattice crosses band_lo, else band_hi; difference marks band samples that
 * the model does not hold, as the reference's kernel does. */
gcm_status gcm_csg_retain_band(gcm_ctx* ctx, gcm_csg_point* d_acc, const float* d_lattice, uint32_t nx, uint32_t ny,
                               uint32_t nz, float iso, float band_lo, float band_hi, gcm_csg_op op,
                               gcm_stream stream);
/* Gratings::primitive_field (src/lattice_files/Gratings.cu:1695-1735, called
 * at src/main.cu:3394, 3978, 4402): restricts a lattice field to the model
 * before it is normalised and meshed.  fixed: samples the retained model does
 * not hold (record val > -1: outside or never touched) become FLT_MAX;
 * otherwise, dynamic: samples where the live primitive field d_primitive is
 * >= 0 become FLT_MAX; neither: nothing changes.  In place on d_lattice
 * (nx*ny*nz samples, like d_acc and d_primitive). */
gcm_status gcm_lattice_mask(gcm_ctx* ctx, const gcm_csg_point* d_acc, const float* d_primitive, float* d_lattice,
                            uint32_t nx, uint32_t ny, uint32_t nz, int fixed, int dynamic, gcm_stream stream);
/* Mesh of the accumulator, one fused pass (Isosurface::computeIsosurface,
 * src/Isosurface.cu:44-135, with classifyVoxel and
 * generateTriangles_lattice_kernel, src/MarchingCubes_kernel.cu:869-1052,
 * 1865-2200).  d_field NULL: the region mode (make_region: cube index from
 * the sign alone, vertices at the accumulated fractions).  d_field set: the
 * live model, the accumulator combined with that primitive field by op, and
 * vertices from vertexInterp_primitive (src/MarchingCubes_kernel.cu:1640-1672).
 * Normals are cross(v2 - v0, v1 - v0) with w = 0.5, as that kernel writes them.
 * Vertex order, capacity and status rules as gcm_mesh_field; d_acc must be
 * 16-byte aligned. */
gcm_status gcm_mesh_retained(gcm_ctx* ctx, const gcm_csg_point* d_acc, const float* d_field, gcm_csg_op op,
                             const gcm_grid* grid, float iso, float* d_pos, float* d_norm, uint64_t capacity_verts,
                             gcm_counts* h_counts, gcm_stream stream);
/* Counting pass of gcm_mesh_retained. */
gcm_status gcm_count_retained(gcm_ctx* ctx, const gcm_csg_point* d_acc, const float* d_field, gcm_csg_op op,
                              const gcm_grid* grid, float iso, gcm_counts* h_counts, gcm_stream stream);
/* The editor's lattice previews (classifyVoxel and
 * generateTriangles_lattice_kernel with `fixed` or `dynamic` set,
 * src/MarchingCubes_kernel.cu:869-1052, 1865-2200): with d_field (d_acc NULL)
 * a primitive field combined by op with the open band band_lo < lattice <
 * band_hi, vertices by vertexInterp_new (:1728-1790); with d_acc (d_field
 * NULL) the accumulated model combined with that band (its difference keeps
 * lattice < band_lo or > band_hi), vertices by vertexInterp_primitive_one
 * (:1676-1726).  Normals calcNormal(v0, v2, v1) with w = 0.5.  capacity 0
 * counts only. */
gcm_status gcm_mesh_lattice_preview(gcm_ctx* ctx, const gcm_csg_point* d_acc, const float* d_field,
                                    const float* d_lattice, gcm_csg_op op, const gcm_grid* grid, float iso,
                                    float band_lo, float band_hi, float* d_pos, float* d_norm,
                                    uint64_t capacity_verts, gcm_counts* h_counts, gcm_stream stream);

/* ------------------------------------------------- spatially variant lattices */

/* The reference's Fourier-grating lattice (SVL, src/main.cu:3578-3711 and
 * 3904-4030, src/lattice_files/Gratings.cu:100-1050).  Coefficient m of the
 * (2 range + 1)^3 unit-cell Fourier coefficients has frequencies (i, j, k),
 * i fastest then j then k, each in [-range, range]. */
typedef struct gcm_svl_params {
  uint32_t nx, ny, nz;      /* solve (control) grid, at least 4 per axis; the lattice is 2nx x 2ny x 2nz */
  float dx, dy, dz;         /* solve grid spacing (the reference uses 1) */
  uint32_t kind;            /* grating rotation: 'n' none, 'r' round, 'b' bend, 's' sine wave */
  uint32_t period_type;     /* 0 constant, 1 per axis, 2 per sample from d_period (nx*ny*nz floats) */
  float period, period_x, period_y, period_z;
  float lcon, lcon_1;       /* 's': amplitude and frequency of the wave */
  uint32_t sinewave_z;      /* 's': also the z-axis wave term */
  uint32_t range;           /* coefficient range (the reference: 2, i.e. 5^3 coefficients) */
  uint32_t n_coeff;         /* coefficients used, from m = 0 (the reference: 62) */
  uint32_t max_iter;        /* CG step cap, the reference's iter (500) */
  float end_res;            /* CG stop when r.d falls to end_res^2 (the reference: 0.01) */
} gcm_svl_params;

/* Gratings::period_data / set_period_kernel (src/lattice_files/Gratings.cu:
 * 818-860, 1376-1389): the radial period field of the spatially variant
 * lattice on the solve grid, sqrt((u + 1)^2 + (v + 1)^2) of the coordinates
 * u, v across the rotation axis ('z': x and y; 'y': x and z; 'x': z and y),
 * each (i - mean) * d.  The reference's round lattices pass mean = N/2.0 and
 * then map the field in place with gcm_normalise_range(range_lo = N/10,
 * range_span = N/4, integer divisions of N = nx; src/main.cu:3929-3931). */
gcm_status gcm_svl_period_field(gcm_ctx* ctx, float* d_period, uint32_t nx, uint32_t ny, uint32_t nz, float dx,
                                float dy, float dz, float mean_x, float mean_y, float mean_z, char axis,
                                gcm_stream stream);
/* Unit cell of TPMS unit_type (gcm_field_unit_cell) on unit_n^3 samples and its
 * Fourier coefficients c_m = (1/N) sum f e^{-2 pi i (i x/n + j y/n + k z/n)}
 * (what the reference takes from an R2C cuFFT scaled by 1/N,
 * src/main.cu:3578-3700), as (re, im) pairs into d_coeff
 * (2 (2 range + 1)^3 floats). */
gcm_status gcm_svl_coefficients(gcm_ctx* ctx, uint32_t unit_type, uint32_t unit_n, uint32_t range, float* d_coeff,
                                gcm_stream stream);
/* Solves the phase field of each of the first n_coeff coefficients on the
 * solve grid (finding_phi_kernel right-hand side, GPUCG_lattice conjugate
 * gradients with the reference's stopping rule) and adds
 * Re(c_m exp(i phi_m)) sampled on the 2x grid (grating_kernel + svl_kernel)
 * to d_svl (8 nx ny nz floats, x fastest), m = 0 .. n_coeff - 1 in order.
 * All solves run together on the device.  d_phase (optional): the solved
 * phases, n_coeff x nx ny nz floats.  h_iters (optional): each solve's
 * final step count (the reference's FinalIter).  Syncs. */
gcm_status gcm_svl_lattice(gcm_ctx* ctx, const gcm_svl_params* params, const float* d_period, const float* d_coeff,
                           float* d_svl, float* d_phase, uint32_t* h_iters, gcm_stream stream);

/* ---------------------------------------------------------------- batches */

/* Many graded lattices meshed together: one launch evaluates every
 * instance's field, one persistent launch meshes every instance's tiles
 * (a single work list and look-back chain), so the outputs are concatenated
 * in instance order and instance i's mesh is exactly what gcm_mesh_lattice
 * produces for it alone.  No counterpart in the reference, which meshes one
 * grid per call (src/Isosurface.cu:401-486).  Control arrays stay owned by the
 * caller and must outlive the batch. */
typedef struct gcm_batch gcm_batch;
typedef struct gcm_batch_instance {
  gcm_lattice lattice;
  gcm_grid grid;
  float iso;
  uint32_t reserved;
} gcm_batch_instance;

/* Allocates everything the batch needs (fields, tile states, instance tables). */
gcm_status gcm_batch_create(gcm_ctx* ctx, const gcm_batch_instance* h_instances, uint32_t n, gcm_batch** out);
gcm_status gcm_batch_destroy(gcm_batch* batch);
/* Counting pass: per-instance vertex and active-voxel counts (host arrays of
 * n, optional) and totals.  Syncs. */
gcm_status gcm_batch_count(gcm_batch* batch, uint64_t* h_verts, uint64_t* h_active, gcm_counts* h_counts,
                           gcm_stream stream);
/* Fields + fused marching cubes of every instance into one output.
 * d_offsets (n+1 uint64, device): instance i's vertices are
 * [d_offsets[i], d_offsets[i+1]).  d_counts: totals and status.  Allocates
 * nothing and never synchronises (capturable). */
gcm_status gcm_batch_mesh_async(gcm_batch* batch, float* d_pos, float* d_norm, uint64_t capacity_verts,
                                uint64_t* d_offsets, gcm_counts* d_counts, gcm_stream stream);
/* The same launches recorded once into a CUDA graph (per set of buffers and
 * stream) and replayed. */
gcm_status gcm_batch_mesh_graph(gcm_batch* batch, float* d_pos, float* d_norm, uint64_t capacity_verts,
                                uint64_t* d_offsets, gcm_counts* d_counts, gcm_stream stream);
/* Times the fused launch over CTA sizes {128, 256} x tile sizes {1024 ..
 * 8192 voxels} on this batch and keeps the fastest; with cache_path, reuses a
 * recorded choice for the same batch shape and appends new ones.  Writes into
 * the given output buffers while timing. */
gcm_status gcm_batch_tune(gcm_batch* batch, float* d_pos, float* d_norm, uint64_t capacity_verts,
                          const char* cache_path, int* h_threads, uint32_t* h_tile_voxels, gcm_stream stream);
/* Launch shape of the fused kernel for this context's single-grid calls:
 * CTA size (128 or 256) and voxels per tile.  Until it is set, the plain and
 * retained forms use 128 threads x 1024 voxels and the band form 256 x 2048. */
gcm_status gcm_ctx_set_launch_shape(gcm_ctx* ctx, int threads, uint32_t tile_voxels);

/* ----------------------------------------------------------------- server */

/* Mesh request server with continuous batching.  `lanes` worker threads, each
 * with its own context and stream, take requests from a bounded FIFO as soon
 * as one is free and the request's memory can be reserved from a device pool
 * of device_pool_bytes; requests that arrive while others run are admitted as
 * lanes and memory free up, and their work overlaps on the GPU.  Memory is
 * admitted exactly in two passes (field, count, then mesh buffers).  With
 * host_pool_bytes > 0 each mesh is copied into pinned host memory before its
 * result completes (latency = submit -> mesh on the host) and its device
 * memory is returned at once.  No counterpart in the reference (an
 * interactive single-request application). */
typedef struct gcm_server gcm_server;

typedef enum gcm_request_kind {
  GCM_REQUEST_LATTICE = 0, /* graded lattice: lattice + grid */
  GCM_REQUEST_CSG = 1,     /* primitive scene: d_prims, n_prims, frame + grid */
  GCM_REQUEST_FIELD = 2    /* caller-owned device field d_field + grid */
} gcm_request_kind;

/* Host-side fault injection for tests (0 in production). */
enum {
  GCM_FAULT_POOL_ALLOC = 1, /* every fault_param-th device reservation fails (retried 3 times) */
  GCM_FAULT_SLOW_LANE = 2,  /* lane 0 sleeps fault_param ms before each request */
  GCM_FAULT_LANE_DIES = 4   /* lane 0 exits after taking its first request, which is re-queued */
};

typedef struct gcm_server_config {
  int device;
  uint32_t lanes;          /* concurrent requests on the GPU (1..64) */
  uint32_t queue_capacity; /* pending requests before submit returns GCM_ERR_BUSY */
  uint32_t fault_flags;
  uint64_t device_pool_bytes; /* budget for fields and meshes in flight */
  uint64_t host_pool_bytes;   /* pinned host memory for results, 0 = results stay on the device */
  uint32_t fault_param;
  uint32_t reserved;
} gcm_server_config;

typedef struct gcm_request {
  uint32_t kind; /* gcm_request_kind */
  uint32_t n_prims;
  gcm_lattice lattice;          /* GCM_REQUEST_LATTICE: device control arrays (resident) */
  const gcm_primitive* d_prims; /* GCM_REQUEST_CSG */
  gcm_frame frame;              /* GCM_REQUEST_CSG */
  const float* d_field;         /* GCM_REQUEST_FIELD */
  gcm_grid grid;
  float iso;
  uint32_t reserved;
  uint64_t user_tag;
} gcm_request;

typedef struct gcm_result {
  uint64_t ticket;
  uint64_t user_tag;
  int32_t status; /* gcm_status of the request */
  uint32_t lane;
  uint64_t total_verts;
  uint64_t active_voxels;
  const float* pos;  /* mesh (host memory when on_host, else device); valid until gcm_server_release */
  const float* norm;
  uint32_t on_host;
  uint32_t reserved;
  double t_submit, t_start, t_done; /* seconds on the server clock (gcm_server_now) */
} gcm_result;

typedef struct gcm_server_stats {
  uint64_t submitted, completed, rejected, cancelled, failed, requeued, pool_faults;
  uint64_t device_pool_peak, device_pool_used, host_pool_peak;
  uint32_t lanes_alive, pending;
} gcm_server_stats;

gcm_status gcm_server_create(const gcm_server_config* cfg, gcm_server** out);
/* Stops the lanes (running requests finish their current step) and frees the pools. */
gcm_status gcm_server_destroy(gcm_server* server);
/* Non-blocking.  GCM_ERR_BUSY when the queue is full; GCM_ERR_REJECTED when the
 * request's field alone exceeds the device pool (a mesh found too large after
 * counting completes with GCM_ERR_REJECTED). */
gcm_status gcm_server_submit(gcm_server* server, const gcm_request* req, uint64_t* h_ticket);
/* Up to `max` completed results, waiting up to timeout_us for the first. */
gcm_status gcm_server_poll(gcm_server* server, gcm_result* out, uint32_t max, uint32_t* n_out, uint64_t timeout_us);
/* Returns a completed request's memory to the pools. */
gcm_status gcm_server_release(gcm_server* server, uint64_t ticket);
/* Cancels a pending request at once, a running one at its next step. */
gcm_status gcm_server_cancel(gcm_server* server, uint64_t ticket);
gcm_status gcm_server_get_stats(gcm_server* server, gcm_server_stats* out);
double gcm_server_now(const gcm_server* server);
/* Host-only check of the server's range allocator (no GPU needed): op[i] > 0
 * reserves op[i] bytes, op[i] < 0 releases the reservation of operation
 * -op[i]-1; result[i] = offset or -1.  Returns the number of free ranges left. */
int64_t gcm_test_pool_script(uint64_t size, const int64_t* op, int64_t* result, uint32_t n);

/* --------------------------------------------------------------- .obj out */

/* Welds an unshared triangle mesh the way File_output::file_write_obj
 * (src/File_output.cu:5-81) does, on the device: positions quantised to
 * float(int(x*1000)*0.001), one .obj vertex per distinct quantised position
 * numbered (1-based) in order of first occurrence, faces with a repeated
 * vertex dropped, repeated identical faces kept once, faces stored in the
 * reference's written order (a, c, b).  d_vertices gets 3 floats per vertex,
 * d_faces 3 uint32 per face (either may be NULL to count only).  Coordinates
 * must stay within |x| < 1048.576 (GCM_ERR_NOT_SUPPORTED otherwise).  Syncs. */
gcm_status gcm_weld_obj(gcm_ctx* ctx, const float* d_pos, uint64_t nverts, float* d_vertices, uint64_t cap_vertices,
                        uint32_t* d_faces, uint64_t cap_faces, uint64_t* h_nvertices, uint64_t* h_nfaces,
                        gcm_stream stream);
/* Welds on the device and writes the .obj text file byte for byte as
 * file_write_obj writes it (header, "v x y z" lines with %g numbers, two blank
 * lines, " f  a c b" lines).  h_nvertices / h_nfaces are optional. */
gcm_status gcm_write_obj(gcm_ctx* ctx, const float* d_pos, uint64_t nverts, const char* path, uint64_t* h_nvertices,
                         uint64_t* h_nfaces, gcm_stream stream);

/* ----------------------------------------------------- allocation-free form */

/* Fused extraction of a fed field for callers that may not allocate device
 * memory (an application that owns every allocation through its own arena, a
 * stream being captured into a CUDA graph, a real-time loop that cannot take
 * an allocation's synchronisation).  It needs no context: the look-back
 * scratch is a fixed 1 MiB array in the library's device image, present on
 * every GPU that loads the library until the process exits, and nothing is
 * allocated or freed.  The caller passes the field, 16-byte aligned output
 * buffers and a device gcm_counts; works on the current device and is
 * stream-ordered (no host synchronisation).  Results equal gcm_mesh_field's.
 *  - Grids whose tile states do not fit the array (at most 131,056 tiles of
 *    whole voxel rows, grown to up to 96 KB of staged rows) return
 *    GCM_ERR_NOT_SUPPORTED before any launch: cubes up to 907^3 fit, 908^3
 *    and larger are refused.
 *  - Every call shares the array and clears the part it uses first; calls
 *    that overlap on the GPU (other streams, other host threads) race on it,
 *    so serialise them.
 *  - The first call on each device looks up the array's device address
 *    (cudaGetSymbolAddress); make that first call before any stream capture.
 *  - Device-side waits are bounded at 2 s (GCM_ERR_DEVICE_TIMEOUT in
 *    d_counts->status).
 * No counterpart in the reference (its scratch is always caller-allocated). */
gcm_status gcm_mesh_field_noalloc(const float* d_field, const gcm_grid* grid, float iso, float* d_pos, float* d_norm,
                                  uint64_t capacity_verts, gcm_counts* d_counts, gcm_stream stream);

/* ----------------------------------------------------------- test hooks */

/* Exercises the bounded waits of the decoupled look-back: ntiles one-warp
 * tiles of aggregate 1 each, except that tile `stall_tile` never publishes
 * its state, so its successors' waits run out after wait_ns.  d_prefix_out
 * (ntiles uint64, device) receives the prefix each tile used.  Returns
 * GCM_ERR_DEVICE_TIMEOUT when the waits ran out as intended; the kernel
 * always returns and the context stays usable.  No counterpart in the
 * reference (which has no bounded waits). */
gcm_status gcm_test_lookback_stall(gcm_ctx* ctx, uint32_t ntiles, uint32_t stall_tile, uint64_t wait_ns,
                                   uint64_t* d_prefix_out, gcm_stream stream);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif

#ifdef __cplusplus
}
#endif

#endif /* GCM_H_ */
