// Parity harness: runs the reference's own CUDA kernels (device code compiled by
// oracle/ref/build_ref.py into oracle/_ref/*.fatbin) on inputs fed from a job
// file and writes their raw outputs, so fixtures can pin the oracle and this
// project's kernels to what the reference computes on a GB300.
//
// Test infrastructure only.  Host orchestration follows the reference's
// Isosurface::computeIsosurface_lattice (src/Isosurface.cu:401-486): classify,
// exclusive scan of the occupancy flags, compaction, exclusive scan of the vertex
// counts, generate.  Two differences, both deliberate:
//   * the scans are done on the host (plain integer prefix sums, exact); the
//     reference calls thrust::exclusive_scan (src/MarchingCubes_kernel.cu:3198-3203),
//     whose kernels cannot be launched by name;
//   * classify is launched as a plain 1-D grid; the reference's 2-D split
//     (src/Isosurface.cu:53-60) drops voxels above 65535 blocks.
// Texture objects for the tables are built from the reference's own tables.h
// data (tests/golden/ref_tables.bin), as allocateTextures_s does
// (src/MarchingCubes_kernel.cu:24-68).
//
// Build (on the GPU machine):
//   g++ -O2 -std=c++17 oracle/ref/ref_runner.cpp -I/usr/local/cuda/include -lcuda
//       -o oracle/_ref/ref_runner
// Use:  ref_runner <fatbin-dir> <variant sm103a|ptx89> <tables.bin> <job.bin> <out.bin>
#include <cuda.h>

#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

struct U3 { uint32_t x, y, z; };
struct F3 { float x, y, z; };

[[noreturn]] void die(const char* what) {
  std::fprintf(stderr, "ref_runner: %s\n", what);
  std::exit(3);
}

void ck(CUresult r, const char* what) {
  if (r != CUDA_SUCCESS) {
    const char* s = nullptr;
    cuGetErrorString(r, &s);
    std::fprintf(stderr, "ref_runner: %s failed: %s\n", what, s ? s : "?");
    std::exit(4);
  }
}

std::vector<uint8_t> slurp(const std::string& path) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) die(("cannot open " + path).c_str());
  std::fseek(f, 0, SEEK_END);
  long n = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  std::vector<uint8_t> b((size_t)n);
  if (n > 0 && std::fread(b.data(), 1, (size_t)n, f) != (size_t)n) die("short read");
  std::fclose(f);
  return b;
}

struct Reader {
  const std::vector<uint8_t>& b;
  size_t off = 0;
  template <class T> T get() {
    if (off + sizeof(T) > b.size()) die("job file truncated");
    T v;
    std::memcpy(&v, b.data() + off, sizeof(T));
    off += sizeof(T);
    return v;
  }
  template <class T> std::vector<T> arr(size_t n) {
    if (off + n * sizeof(T) > b.size()) die("job file truncated (array)");
    std::vector<T> v(n);
    if (n) std::memcpy(v.data(), b.data() + off, n * sizeof(T));
    off += n * sizeof(T);
    return v;
  }
};

struct Writer {
  FILE* f;
  template <class T> void put(T v) { std::fwrite(&v, sizeof(T), 1, f); }
  template <class T> void arr(const std::vector<T>& v) {
    if (!v.empty()) std::fwrite(v.data(), sizeof(T), v.size(), f);
  }
};

// Finds a kernel by its unmangled name inside a loaded module: the Itanium
// mangling of a free function starts with _Z<len><name>.
CUfunction find_kernel(CUmodule mod, const char* name) {
  unsigned n = 0;
  ck(cuModuleGetFunctionCount(&n, mod), "cuModuleGetFunctionCount");
  std::vector<CUfunction> fs(n);
  ck(cuModuleEnumerateFunctions(fs.data(), n, mod), "cuModuleEnumerateFunctions");
  std::string key = "_Z" + std::to_string(std::strlen(name)) + name;
  for (CUfunction f : fs) {
    const char* nm = nullptr;
    ck(cuFuncGetName(&nm, f), "cuFuncGetName");
    if (nm && std::strncmp(nm, key.c_str(), key.size()) == 0) return f;
  }
  die((std::string("kernel not found: ") + name).c_str());
}

template <class T> CUdeviceptr dalloc(size_t n, int fill_byte = 0) {
  CUdeviceptr p = 0;
  size_t bytes = (n ? n : 1) * sizeof(T);
  ck(cuMemAlloc(&p, bytes), "cuMemAlloc");
  ck(cuMemsetD8(p, (unsigned char)fill_byte, bytes), "cuMemsetD8");
  return p;
}

template <class T> CUdeviceptr dupload(const std::vector<T>& v, size_t pad_to = 0) {
  size_t n = v.size() > pad_to ? v.size() : pad_to;
  CUdeviceptr p = dalloc<T>(n);
  if (!v.empty()) ck(cuMemcpyHtoD(p, v.data(), v.size() * sizeof(T)), "cuMemcpyHtoD");
  return p;
}

template <class T> std::vector<T> ddownload(CUdeviceptr p, size_t n) {
  std::vector<T> v(n);
  if (n) ck(cuMemcpyDtoH(v.data(), p, n * sizeof(T)), "cuMemcpyDtoH");
  return v;
}

CUtexObject make_u32_tex(CUdeviceptr p, size_t count) {
  CUDA_RESOURCE_DESC rd;
  std::memset(&rd, 0, sizeof(rd));
  rd.resType = CU_RESOURCE_TYPE_LINEAR;
  rd.res.linear.devPtr = p;
  rd.res.linear.format = CU_AD_FORMAT_UNSIGNED_INT32;
  rd.res.linear.numChannels = 1;
  rd.res.linear.sizeInBytes = count * sizeof(uint32_t);
  CUDA_TEXTURE_DESC td;
  std::memset(&td, 0, sizeof(td));
  td.addressMode[0] = CU_TR_ADDRESS_MODE_CLAMP;
  td.filterMode = CU_TR_FILTER_MODE_POINT;
  td.flags = CU_TRSF_READ_AS_INTEGER;
  CUtexObject t = 0;
  ck(cuTexObjectCreate(&t, &rd, &td, nullptr), "cuTexObjectCreate");
  return t;
}

void launch(CUfunction f, unsigned gx, unsigned gy, unsigned gz, unsigned bx, unsigned by,
            unsigned bz, void** args) {
  ck(cuLaunchKernel(f, gx, gy, gz, bx, by, bz, 0, nullptr, args, nullptr), "cuLaunchKernel");
  ck(cuCtxSynchronize(), "cuCtxSynchronize");
}

unsigned blocks_for(uint64_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

std::vector<uint32_t> exclusive_scan(const std::vector<uint32_t>& in) {
  std::vector<uint32_t> out(in.size());
  uint32_t acc = 0;
  for (size_t i = 0; i < in.size(); ++i) { out[i] = acc; acc += in[i]; }
  return out;
}

struct Tables {
  CUdeviceptr tri = 0, nverts = 0;
  CUtexObject tri_tex = 0, nverts_tex = 0;
};

Tables load_tables(const std::string& path) {
  auto b = slurp(path);
  if (b.size() != 512 + 4096 + 256) die("tables file has the wrong size");
  std::vector<uint32_t> tri(4096), nv(256);
  for (int i = 0; i < 4096; ++i) tri[i] = b[512 + i];
  for (int i = 0; i < 256; ++i) nv[i] = b[4608 + i];
  Tables t;
  t.tri = dupload(tri);
  t.nverts = dupload(nv);
  t.tri_tex = make_u32_tex(t.tri, 4096);
  t.nverts_tex = make_u32_tex(t.nverts, 256);
  return t;
}

// Classify + compact, shared by the plain and band cases.  The classify field
// `vol` is the one whose `< iso` test makes the cube index (classifyVoxel_new,
// src/MarchingCubes_kernel.cu:3207-3249).
struct Classified {
  uint32_t nvox = 0, active = 0, total = 0;
  std::vector<uint32_t> verts, occ, occ_scan, verts_scan, compacted;
  CUdeviceptr d_verts_scan = 0, d_compacted = 0;
};

Classified classify_and_compact(CUmodule mc, const Tables& T, CUdeviceptr vol, U3 gsize, float iso) {
  Classified c;
  U3 mask{gsize.x - 1, gsize.y - 1, gsize.z - 1};
  U3 shift{1, gsize.x - 1, (gsize.x - 1) * (gsize.y - 1)};
  c.nvox = mask.x * mask.y * mask.z;
  CUdeviceptr d_verts = dalloc<uint32_t>(c.nvox), d_occ = dalloc<uint32_t>(c.nvox);
  F3 vs{1.f, 1.f, 1.f};
  CUfunction k_cls = find_kernel(mc, "classifyVoxel_new");
  {
    void* a[] = {&d_verts, &d_occ, &vol, &gsize, &shift, &mask, &c.nvox, &vs, &iso,
                 const_cast<CUtexObject*>(&T.nverts_tex)};
    launch(k_cls, blocks_for(c.nvox, 1024), 1, 1, 1024, 1, 1, a);
  }
  c.verts = ddownload<uint32_t>(d_verts, c.nvox);
  c.occ = ddownload<uint32_t>(d_occ, c.nvox);
  c.occ_scan = exclusive_scan(c.occ);
  c.verts_scan = exclusive_scan(c.verts);
  c.active = c.nvox ? c.occ_scan.back() + c.occ.back() : 0;
  c.total = c.nvox ? c.verts_scan.back() + c.verts.back() : 0;
  CUdeviceptr d_occ_scan = dupload(c.occ_scan);
  c.d_compacted = dalloc<uint32_t>(c.active ? c.active : 1);
  CUfunction k_cmp = find_kernel(mc, "compactVoxels");
  {
    void* a[] = {&c.d_compacted, &d_occ, &d_occ_scan, &c.nvox};
    launch(k_cmp, blocks_for(c.nvox, 1024), 1, 1, 1024, 1, 1, a);
  }
  c.compacted = ddownload<uint32_t>(c.d_compacted, c.active);
  c.d_verts_scan = dupload(c.verts_scan);
  cuMemFree(d_verts);
  cuMemFree(d_occ);
  cuMemFree(d_occ_scan);
  return c;
}

void write_classified(Writer& w, const Classified& c) {
  w.put<uint32_t>(c.nvox);
  w.put<uint32_t>(c.active);
  w.put<uint32_t>(c.total);
  w.arr(c.verts);
  w.arr(c.occ);
  w.arr(c.occ_scan);
  w.arr(c.verts_scan);
  w.arr(c.compacted);
}

// kind 1: plain marching cubes on a fed field.  generateTriangles_lattice_kernel_3
// (src/MarchingCubes_kernel.cu:3041-3170) takes its cube index as
// (f < iso) && (f > 0); jobs feed strictly positive fields so it equals the
// classify index.
void run_mc_plain(Reader& r, Writer& w, CUmodule mc, const Tables& T) {
  U3 g{r.get<uint32_t>(), r.get<uint32_t>(), r.get<uint32_t>()};
  float iso = r.get<float>();
  F3 vs{r.get<float>(), r.get<float>(), r.get<float>()};
  F3 gc{r.get<float>(), r.get<float>(), r.get<float>()};
  auto field = r.arr<float>((size_t)g.x * g.y * g.z);
  CUdeviceptr d_field = dupload(field);
  Classified c = classify_and_compact(mc, T, d_field, g, iso);
  uint32_t maxv = c.total + 16;
  CUdeviceptr d_pos = dalloc<float>(4ull * maxv, 0xFF), d_norm = dalloc<float>(4ull * maxv, 0xFF);
  U3 mask{g.x - 1, g.y - 1, g.z - 1};
  U3 shift{1, g.x - 1, (g.x - 1) * (g.y - 1)};
  if (c.active) {
    CUfunction k = find_kernel(mc, "generateTriangles_lattice_kernel_3");
    void* a[] = {&d_pos, &d_norm, &c.d_compacted, &c.d_verts_scan, &g, &shift, &mask, &vs, &gc,
                 &iso, &c.active, &maxv, const_cast<CUtexObject*>(&T.tri_tex),
                 const_cast<CUtexObject*>(&T.nverts_tex), &c.total, &d_field, &iso};
    launch(k, blocks_for(c.active, 32), 1, 1, 32, 1, 1, a);
  }
  write_classified(w, c);
  w.arr(ddownload<float>(d_pos, 4ull * c.total));
  w.arr(ddownload<float>(d_norm, 4ull * c.total));
  cuMemFree(d_field); cuMemFree(d_pos); cuMemFree(d_norm);
  cuMemFree(c.d_compacted); cuMemFree(c.d_verts_scan);
}

// kind 2: band-mode marching cubes.  Cube index from a 0/1 label field, vertices
// from the normalised field with the band edges (generateTriangles_lattice_kernel_newone,
// src/MarchingCubes_kernel.cu:3678-3817).  Also runs the two-field variant
// (generateTriangles_lattice_kernel_new, :3424-3570) with the arguments
// spatial_lattice_run passes (src/main.cu:4006-4010: iso1 = iso2 = 0).
void run_mc_band(Reader& r, Writer& w, CUmodule mc, const Tables& T) {
  U3 g{r.get<uint32_t>(), r.get<uint32_t>(), r.get<uint32_t>()};
  float iso = r.get<float>(), b1 = r.get<float>(), b2 = r.get<float>();
  F3 vs{r.get<float>(), r.get<float>(), r.get<float>()};
  F3 gc{r.get<float>(), r.get<float>(), r.get<float>()};
  size_t P = (size_t)g.x * g.y * g.z;
  auto label = r.arr<float>(P);
  auto normf = r.arr<float>(P);
  CUdeviceptr d_label = dupload(label), d_normf = dupload(normf), d_two = dupload(normf);
  Classified c = classify_and_compact(mc, T, d_label, g, iso);
  uint32_t maxv = c.total + 16;
  U3 mask{g.x - 1, g.y - 1, g.z - 1};
  U3 shift{1, g.x - 1, (g.x - 1) * (g.y - 1)};
  write_classified(w, c);
  for (int variant = 0; variant < 2; ++variant) {
    CUdeviceptr d_pos = dalloc<float>(4ull * maxv, 0xFF), d_norm = dalloc<float>(4ull * maxv, 0xFF);
    if (c.active) {
      if (variant == 0) {
        CUfunction k = find_kernel(mc, "generateTriangles_lattice_kernel_newone");
        void* a[] = {&d_pos, &d_norm, &c.d_compacted, &c.d_verts_scan, &d_label, &g, &shift, &mask,
                     &vs, &gc, &iso, &c.active, &maxv, const_cast<CUtexObject*>(&T.tri_tex),
                     const_cast<CUtexObject*>(&T.nverts_tex), &c.total, &d_normf, &b1, &b2};
        launch(k, blocks_for(c.active, 32), 1, 1, 32, 1, 1, a);
      } else {
        float z0 = 0.f, z1 = 0.f;
        CUfunction k = find_kernel(mc, "generateTriangles_lattice_kernel_new");
        void* a[] = {&d_pos, &d_norm, &c.d_compacted, &c.d_verts_scan, &d_label, &g, &shift, &mask,
                     &vs, &gc, &iso, &c.active, &maxv, const_cast<CUtexObject*>(&T.tri_tex),
                     const_cast<CUtexObject*>(&T.nverts_tex), &c.total, &d_normf, &d_two, &b1, &b2,
                     &z0, &z1};
        launch(k, blocks_for(c.active, 32), 1, 1, 32, 1, 1, a);
      }
    }
    w.arr(ddownload<float>(d_pos, 4ull * c.total));
    w.arr(ddownload<float>(d_norm, 4ull * c.total));
    cuMemFree(d_pos); cuMemFree(d_norm);
  }
  cuMemFree(d_label); cuMemFree(d_normf); cuMemFree(d_two);
  cuMemFree(c.d_compacted); cuMemFree(c.d_verts_scan);
}

// kind 3: TPMS unit cell (create_lattice_kernel, src/lattice_files/Fft_lattice.cu:11-93),
// launched with the reference's 16x8x8 blocks (:95-98).
void run_unit_cell(Reader& r, Writer& w, CUmodule fft) {
  uint32_t nx = r.get<uint32_t>(), ny = r.get<uint32_t>(), nz = r.get<uint32_t>(), type = r.get<uint32_t>();
  // The kernel calls __syncthreads() inside its bounds check; sizes that tile the
  // 16x8x8 blocks exactly keep every thread of a block on the same path.
  if (nx % 16 || ny % 8 || nz % 8) die("unit-cell jobs must tile the 16x8x8 blocks exactly");
  uint32_t size = nx * ny * nz;
  CUdeviceptr d = dalloc<float>(size);
  CUfunction k = find_kernel(fft, "create_lattice_kernel");
  void* a[] = {&d, &nx, &ny, &nz, &size, &type};
  launch(k, (nx + 15) / 16, (ny + 7) / 8, (nz + 7) / 8, 16, 8, 8, a);
  w.arr(ddownload<float>(d, size));
  cuMemFree(d);
}

// kind 4: primitive fields (src/Modelling.cu:244-750), 1-D launches of 1024
// threads.  Three of the kernels (cuboid, cuboid shell, pyramid frustum) have no
// bounds check, so the output buffer is padded to the whole launch.
void run_primitive(Reader& r, Writer& w, CUmodule mdl) {
  uint32_t prim = r.get<uint32_t>();
  int nx = r.get<int32_t>(), ny = r.get<int32_t>(), nz = r.get<int32_t>();
  float dx = r.get<float>(), dy = r.get<float>(), dz = r.get<float>();
  F3 center{r.get<float>(), r.get<float>(), r.get<float>()};
  F3 v3{r.get<float>(), r.get<float>(), r.get<float>()};  // axis or Euler angles
  float p[6];
  for (float& x : p) x = r.get<float>();
  uint32_t flag = r.get<uint32_t>();
  size_t P = (size_t)nx * ny * nz;
  unsigned blocks = blocks_for(P, 1024);
  CUdeviceptr d = dalloc<float>((size_t)blocks * 1024);
  bool sel = flag != 0;
  CUfunction k;
  switch (prim) {
    case 0: {  // implicit_sphere_kernel(data, center, radius, thickness, Nx,Ny,Nz, dx,dy,dz, shell)
      k = find_kernel(mdl, "implicit_sphere_kernel");
      void* a[] = {&d, &center, &p[0], &p[1], &nx, &ny, &nz, &dx, &dy, &dz, &sel};
      launch(k, blocks, 1, 1, 1024, 1, 1, a);
      break;
    }
    case 1: {  // distance_from_line_kernel(data, center, axis, radius, t_radial, t_axial, Nx..dz, disc)
      k = find_kernel(mdl, "distance_from_line_kernel");
      void* a[] = {&d, &center, &v3, &p[0], &p[1], &p[2], &nx, &ny, &nz, &dx, &dy, &dz, &sel};
      launch(k, blocks, 1, 1, 1024, 1, 1, a);
      break;
    }
    case 2: {  // implicit_cuboid_kernel(data, center, angles, xw, yw, zw, Nx..dz)
      k = find_kernel(mdl, "implicit_cuboid_kernel");
      void* a[] = {&d, &center, &v3, &p[0], &p[1], &p[2], &nx, &ny, &nz, &dx, &dy, &dz};
      launch(k, blocks, 1, 1, 1024, 1, 1, a);
      break;
    }
    case 3: {  // implicit_cuboid_shell_kernel(data, center, angles, xw, yw, zw, thickness, Nx..dz)
      k = find_kernel(mdl, "implicit_cuboid_shell_kernel");
      void* a[] = {&d, &center, &v3, &p[0], &p[1], &p[2], &p[3], &nx, &ny, &nz, &dx, &dy, &dz};
      launch(k, blocks, 1, 1, 1024, 1, 1, a);
      break;
    }
    case 4: {  // implicit_torus_kernel(data, center, angles, R, r, Nx..dz)
      k = find_kernel(mdl, "implicit_torus_kernel");
      void* a[] = {&d, &center, &v3, &p[0], &p[1], &nx, &ny, &nz, &dx, &dy, &dz};
      launch(k, blocks, 1, 1, 1024, 1, 1, a);
      break;
    }
    case 5: {  // implicit_cone_kernel(data, center, angles, base_radius, height, Nx..dz)
      k = find_kernel(mdl, "implicit_cone_kernel");
      void* a[] = {&d, &center, &v3, &p[0], &p[1], &nx, &ny, &nz, &dx, &dy, &dz};
      launch(k, blocks, 1, 1, 1024, 1, 1, a);
      break;
    }
    case 6: {  // implicit_cone_frustum_kernel(data, center, angles, top_r, bottom_r, height, Nx..dz)
      k = find_kernel(mdl, "implicit_cone_frustum_kernel");
      void* a[] = {&d, &center, &v3, &p[0], &p[1], &p[2], &nx, &ny, &nz, &dx, &dy, &dz};
      launch(k, blocks, 1, 1, 1024, 1, 1, a);
      break;
    }
    case 7: {  // implicit_pyramid_frustum_kernel(data, center, angles, xb, xt, yh, zb, zt, Nx..dz)
      k = find_kernel(mdl, "implicit_pyramid_frustum_kernel");
      void* a[] = {&d, &center, &v3, &p[0], &p[1], &p[2], &p[3], &p[4], &nx, &ny, &nz, &dx, &dy, &dz};
      launch(k, blocks, 1, 1, 1024, 1, 1, a);
      break;
    }
    default:
      die("unknown primitive");
  }
  w.arr(ddownload<float>(d, P));
  cuMemFree(d);
}

// kind 5: band normalisation (GPU_buffer_normalise_four,
// src/lattice_files/Gratings.cu:1579-1617).  Jobs use sizes that are multiples of
// 1024: the first reduction kernel leaves the tail of a partial block unset.
void run_normalise_four(Reader& r, Writer& w, CUmodule gr) {
  int nx = r.get<int32_t>(), ny = r.get<int32_t>(), nz = r.get<int32_t>();
  float i1 = r.get<float>(), i2 = r.get<float>();
  size_t P = (size_t)nx * ny * nz;
  auto data = r.arr<float>(P);
  int n = (int)P;
  int block_num = (int)blocks_for(P, 1024);
  CUdeviceptr d_in = dupload(data), d_red = dalloc<float>(2 * (size_t)block_num);
  CUdeviceptr d_label = dalloc<float>(P), d_norm = dalloc<float>(P);
  {
    CUfunction k = find_kernel(gr, "GPUScalar_normalise_kernel_lattice");
    void* a[] = {&d_red, &d_in, &n};
    launch(k, (unsigned)block_num, 1, 1, 1024, 1, 1, a);
  }
  {
    CUfunction k = find_kernel(gr, "Min_reduction_lattice");
    void* a[] = {&d_red, &block_num};
    launch(k, 1, 1, 1, 1024, 1, 1, a);
  }
  float mm[2];
  ck(cuMemcpyDtoH(mm, d_red, sizeof(mm)), "cuMemcpyDtoH");
  {
    CUfunction k = find_kernel(gr, "device_bufferfour");
    void* a[] = {&d_in, &d_label, &d_norm, &mm[0], &mm[1], &nx, &ny, &nz, &i1, &i2};
    launch(k, (unsigned)block_num, 1, 1, 1024, 1, 1, a);
  }
  w.put<float>(mm[0]);
  w.put<float>(mm[1]);
  w.arr(ddownload<float>(d_label, P));
  w.arr(ddownload<float>(d_norm, P));
  cuMemFree(d_in); cuMemFree(d_red); cuMemFree(d_label); cuMemFree(d_norm);
}

// kind 11: the SVL period field, Gratings::period_data (src/lattice_files/
// Gratings.cu:1376-1389: set_period_kernel :818-860) then
// GPU_buffer_normalise_three (:1539-1572: GPUScalar_normalise_kernel_lattice,
// Min_reduction_lattice, device_bufferthree :1071-1087) in place, as
// src/main.cu:3929-3931 calls them.  set_period_kernel synchronises inside its
// bounds test, so jobs cover whole 1024-thread blocks (the runner refuses
// others).  Writes the raw field, the min/max pair and the mapped field.
void run_period(Reader& r, Writer& w, CUmodule gr) {
  int nx = r.get<int32_t>(), ny = r.get<int32_t>(), nz = r.get<int32_t>();
  float dx = r.get<float>(), dy = r.get<float>(), dz = r.get<float>();
  float mx = r.get<float>(), my = r.get<float>(), mz = r.get<float>();
  char axis = (char)r.get<uint32_t>();
  float a1 = r.get<float>(), b1 = r.get<float>();
  size_t P = (size_t)nx * ny * nz;
  if (P % 1024) die("period jobs must fill whole 1024-thread blocks");
  int n = (int)P;
  int block_num = (int)blocks_for(P, 1024);
  CUdeviceptr d_p = dalloc<float>(P), d_red = dalloc<float>(2 * (size_t)block_num);
  {
    CUfunction k = find_kernel(gr, "set_period_kernel");
    void* a[] = {&d_p, &nx, &ny, &nz, &dx, &dy, &dz, &mx, &my, &mz, &axis};
    launch(k, (unsigned)block_num, 1, 1, 1024, 1, 1, a);
  }
  w.arr(ddownload<float>(d_p, P));
  {
    CUfunction k = find_kernel(gr, "GPUScalar_normalise_kernel_lattice");
    void* a[] = {&d_red, &d_p, &n};
    launch(k, (unsigned)block_num, 1, 1, 1024, 1, 1, a);
  }
  {
    CUfunction k = find_kernel(gr, "Min_reduction_lattice");
    void* a[] = {&d_red, &block_num};
    launch(k, 1, 1, 1, 1024, 1, 1, a);
  }
  float mm[2];
  ck(cuMemcpyDtoH(mm, d_red, sizeof(mm)), "cuMemcpyDtoH");
  {
    CUfunction k = find_kernel(gr, "device_bufferthree");
    void* a[] = {&d_p, &d_p, &n, &mm[0], &mm[1], &a1, &b1};
    launch(k, (unsigned)block_num, 1, 1, 1024, 1, 1, a);
  }
  w.put<float>(mm[0]);
  w.put<float>(mm[1]);
  w.arr(ddownload<float>(d_p, P));
  cuMemFree(d_p); cuMemFree(d_red);
}

// kind 12: Gratings::primitive_field (src/lattice_files/Gratings.cu:1695-1735):
// primitive_field_kernel sets the lattice to FLT_MAX where the retained model
// (fixed) or the live primitive field (dynamic) leaves a sample out.  Inputs:
// the fixed / dynamic flags, the grid_points accumulator (16-byte records), the
// primitive field and the lattice; writes the lattice after the kernel.
void run_mask(Reader& r, Writer& w, CUmodule gr) {
  uint32_t n = r.get<uint32_t>();
  bool fixed = r.get<uint32_t>() != 0, dynamic = r.get<uint32_t>() != 0;
  auto acc = r.arr<uint8_t>(16 * (size_t)n);
  auto prim = r.arr<float>(n);
  auto lat = r.arr<float>(n);
  CUdeviceptr d_acc = dupload(acc), d_prim = dupload(prim), d_lat = dupload(lat);
  float isoval = 0.0f;
  unsigned int size = n;
  CUfunction k = find_kernel(gr, "primitive_field_kernel");
  void* a[] = {&d_acc, &d_prim, &d_lat, &isoval, &size, &fixed, &dynamic};
  launch(k, (unsigned)blocks_for(n, 1024), 1, 1, 1024, 1, 1, a);
  w.arr(ddownload<float>(d_lat, n));
  cuMemFree(d_acc); cuMemFree(d_prim); cuMemFree(d_lat);
}

}  // namespace

// kind 7: retained primitive editing.  A zeroed grid_points accumulator
// (src/MarchingCubes_kernel.h:12-18) folds a sequence of primitive fields with
// classify_copy_Voxel as Isosurface::copy_parameter launches it
// (src/Isosurface.cu:16-27, static mode); then the accumulator is meshed as
// Isosurface::computeIsosurface does (src/Isosurface.cu:44-135): classifyVoxel,
// scans, compactVoxels, generateTriangles_lattice_kernel, in the make_region
// mode (mode 0) or the plain primitive mode with one more primitive field
// (mode 1).  Unused field arguments get zeroed buffers (the kernels read them).
// kind 10 is kind 7 with, per fold, the mode (0 static, 1 lattice band) and
// the band edges iso1, iso2 before the field; a band fold passes the field as
// classify_copy_Voxel's vol_lattice with dynamic = true.
void run_retain(Reader& r, Writer& w, CUmodule mc, const Tables& T, bool banded) {
  U3 g{r.get<uint32_t>(), r.get<uint32_t>(), r.get<uint32_t>()};
  float iso = r.get<float>();
  F3 vs{r.get<float>(), r.get<float>(), r.get<float>()};
  F3 gc{r.get<float>(), r.get<float>(), r.get<float>()};
  const size_t P = (size_t)g.x * g.y * g.z;
  U3 mask{g.x - 1, g.y - 1, g.z - 1};
  U3 shift{1, g.x - 1, (g.x - 1) * (g.y - 1)};
  uint32_t nvox = mask.x * mask.y * mask.z;
  CUdeviceptr d_acc = dalloc<uint8_t>(16 * P), d_zero = dalloc<float>(P), d_verts = dalloc<uint32_t>(nvox);
  uint32_t n_folds = r.get<uint32_t>();
  CUfunction k_fold = find_kernel(mc, "classify_copy_Voxel");
  for (uint32_t i = 0; i < n_folds; ++i) {
    uint32_t op = r.get<uint32_t>();
    bool dynamic = false;
    float iso1 = 0.0f, iso2 = 0.0f;
    if (banded) {
      dynamic = r.get<uint32_t>() != 0;
      iso1 = r.get<float>();
      iso2 = r.get<float>();
    }
    auto f = r.arr<float>(P);
    CUdeviceptr d_f = dupload(f);
    bool fixed = false, ou = op == 0, od = op == 1, oi = op == 2;
    CUdeviceptr d_two = dynamic ? d_zero : d_f, d_lat = dynamic ? d_f : d_zero;
    void* a[] = {&d_verts, &d_acc, &d_two, &d_lat, &fixed, &dynamic, &iso1, &iso2, &g, &shift, &mask, &nvox,
                 &vs, &iso, const_cast<CUtexObject*>(&T.nverts_tex), &ou, &od, &oi};
    launch(k_fold, blocks_for(P, 1024), 1, 1, 1024, 1, 1, a);
    cuMemFree(d_f);
  }
  // mesh mode: 0 region, 1 primitive preview (field), and in kind 10 also
  // 2 lattice "fixed" (band edges, field, lattice) and 3 lattice "dynamic"
  // (band edges, lattice): classifyVoxel / generateTriangles_lattice_kernel
  // with fixed or dynamic set
  uint32_t mode = r.get<uint32_t>(), pop = r.get<uint32_t>();
  float iso1 = 0.0f, iso2 = 0.0f;
  if (banded && mode >= 2) {
    iso1 = r.get<float>();
    iso2 = r.get<float>();
  }
  CUdeviceptr d_dyn = d_zero, d_lat = d_zero;
  if (mode == 1 || mode == 2) d_dyn = dupload(r.arr<float>(P));
  if (banded && mode >= 2) d_lat = dupload(r.arr<float>(P));
  bool ou = pop == 0, od = pop == 1, oi = pop == 2, prim = mode <= 1, topo = false, lat = mode >= 2,
       fixed = mode == 2, dynamic = mode == 3, region = mode == 0;
  CUdeviceptr d_occ = dalloc<uint32_t>(nvox);
  CUfunction k_cls = find_kernel(mc, "classifyVoxel");
  {
    void* a[] = {&d_zero, &g, &d_verts, &d_occ, &d_acc, &d_dyn, &d_zero, &d_lat, &g, &shift, &mask, &nvox,
                 &iso1, &iso2, &vs, &iso, const_cast<CUtexObject*>(&T.nverts_tex), &ou, &od, &oi, &prim, &topo,
                 &lat, &fixed, &dynamic, &region};
    launch(k_cls, blocks_for(nvox, 1024), 1, 1, 1024, 1, 1, a);
  }
  Classified c;
  c.nvox = nvox;
  c.verts = ddownload<uint32_t>(d_verts, nvox);
  c.occ = ddownload<uint32_t>(d_occ, nvox);
  c.occ_scan = exclusive_scan(c.occ);
  c.verts_scan = exclusive_scan(c.verts);
  c.active = nvox ? c.occ_scan.back() + c.occ.back() : 0;
  c.total = nvox ? c.verts_scan.back() + c.verts.back() : 0;
  CUdeviceptr d_occ_scan = dupload(c.occ_scan);
  c.d_compacted = dalloc<uint32_t>(c.active ? c.active : 1);
  CUfunction k_cmp = find_kernel(mc, "compactVoxels");
  {
    void* a[] = {&c.d_compacted, &d_occ, &d_occ_scan, &nvox};
    launch(k_cmp, blocks_for(nvox, 1024), 1, 1, 1024, 1, 1, a);
  }
  c.compacted = ddownload<uint32_t>(c.d_compacted, c.active);
  c.d_verts_scan = dupload(c.verts_scan);
  uint32_t maxv = c.total + 16;
  CUdeviceptr d_pos = dalloc<float>(4ull * maxv, 0xFF), d_norm = dalloc<float>(4ull * maxv, 0xFF);
  if (c.active) {
    CUfunction k = find_kernel(mc, "generateTriangles_lattice_kernel");
    void* a[] = {&d_pos, &d_norm, &c.d_compacted, &c.d_verts_scan, &g, &shift, &mask, &vs, &gc, &iso,
                 &c.active, &maxv, const_cast<CUtexObject*>(&T.tri_tex), const_cast<CUtexObject*>(&T.nverts_tex),
                 &c.total, &d_acc, &d_dyn, &d_zero, &d_lat, &iso1, &iso2, &d_verts, &ou, &od, &oi, &prim, &topo,
                 &lat, &fixed, &dynamic, &region};
    launch(k, blocks_for(c.active, 32), 1, 1, 32, 1, 1, a);
  }
  w.arr(ddownload<uint8_t>(d_acc, 16 * P));
  write_classified(w, c);
  w.arr(ddownload<float>(d_pos, 4ull * c.total));
  w.arr(ddownload<float>(d_norm, 4ull * c.total));
  if (d_dyn != d_zero) cuMemFree(d_dyn);
  if (d_lat != d_zero) cuMemFree(d_lat);
  cuMemFree(d_acc); cuMemFree(d_zero); cuMemFree(d_verts); cuMemFree(d_occ); cuMemFree(d_occ_scan);
  cuMemFree(d_pos); cuMemFree(d_norm); cuMemFree(c.d_compacted); cuMemFree(c.d_verts_scan);
}

// kind 8: the reference's spatially variant lattice (src/main.cu:3904-4030):
// for coefficient m = 0 .. n-1 finding_phi_kernel, GPUCG_lattice (its host loop
// restated, its kernels launched as it launches them, Gratings.cu:875-974),
// the phase copied into a 3-D float array read through a linear-filtered
// texture with the reference's descriptor (Interpolations.cu:79-107),
// grating_kernel and svl_kernel.  Writes per m the right-hand side, the phase
// and the step count, then the accumulated lattice.  The coefficients are an
// input (the reference takes them from cuFFT).  Kind 9: the same run timed
// (wall clock over the coefficient loop, nothing downloaded but the step counts).
void run_svl(Reader& r, Writer& w, CUmodule gr, bool timing) {
  int X = r.get<int32_t>(), Y = r.get<int32_t>(), Z = r.get<int32_t>();
  float dx = r.get<float>(), dy = r.get<float>(), dz = r.get<float>();
  char kind = (char)r.get<uint32_t>();
  int ptype = r.get<int32_t>();
  float per = r.get<float>(), px = r.get<float>(), py = r.get<float>(), pz = r.get<float>();
  float lcon = r.get<float>(), lcon1 = r.get<float>();
  bool sinez = r.get<uint32_t>() != 0;
  int range = r.get<int32_t>();
  uint32_t n = r.get<uint32_t>(), max_iter = r.get<uint32_t>();
  float end_res = r.get<float>();
  const size_t P = (size_t)X * Y * Z;
  auto period = r.arr<float>(P);
  const int wdt = 2 * range + 1;
  auto coef = r.arr<float>(2 * (size_t)wdt * wdt * wdt);
  CUdeviceptr d_phi = dalloc<float>(P), d_per = dupload(period), d_d = dalloc<float>(P), d_q = dalloc<float>(P),
              d_res = dalloc<float>(P), d_coef = dupload(coef), d_svl = dalloc<float>(8 * P),
              d_ga = dalloc<float>(16 * P);
  const int nb = (int)(P / 1024) + ((P % 1024) ? 1 : 0);
  CUdeviceptr d_red = dalloc<float>((size_t)nb);
  CUDA_ARRAY3D_DESCRIPTOR ad;
  std::memset(&ad, 0, sizeof(ad));
  ad.Width = X; ad.Height = Y; ad.Depth = Z; ad.Format = CU_AD_FORMAT_FLOAT; ad.NumChannels = 1;
  CUarray arr;
  ck(cuArray3DCreate(&arr, &ad), "cuArray3DCreate");
  CUDA_RESOURCE_DESC rd;
  std::memset(&rd, 0, sizeof(rd));
  rd.resType = CU_RESOURCE_TYPE_ARRAY;
  rd.res.array.hArray = arr;
  CUDA_TEXTURE_DESC td;
  std::memset(&td, 0, sizeof(td));
  td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = CU_TR_ADDRESS_MODE_WRAP;
  td.filterMode = CU_TR_FILTER_MODE_LINEAR;
  CUtexObject tex = 0;
  ck(cuTexObjectCreate(&tex, &rd, &td, nullptr), "cuTexObjectCreate");
  CUfunction k_phi = find_kernel(gr, "finding_phi_kernel"), k_mv = find_kernel(gr, "GPUMatvec_lattice_kernel"),
             k_sc = find_kernel(gr, "GPUScalar_lattice_kernel"), k_red = find_kernel(gr, "Reduction_lattice"),
             k_ax = find_kernel(gr, "VecSMultAddKernel_lattice"), k_gr = find_kernel(gr, "grating_kernel"),
             k_svl = find_kernel(gr, "svl_kernel");
  int Pi = (int)P;
  const unsigned g1 = blocks_for(P, 1024);
  auto dot = [&](CUdeviceptr a, CUdeviceptr b) {
    void* as[] = {&d_red, &a, &b, &Pi};
    launch(k_sc, g1, 1, 1, 1024, 1, 1, as);
    void* ar[] = {&d_red, &d_red, const_cast<int*>(&nb)};
    launch(k_red, 1, 1, 1, 1024, 1, 1, ar);
    float v = 0;
    ck(cuMemcpyDtoH(&v, d_red, sizeof(float)), "cuMemcpyDtoH");
    ck(cuMemsetD8(d_red, 0, sizeof(float) * nb), "cuMemsetD8");
    return v;
  };
  auto axpby = [&](CUdeviceptr v, float a1, CUdeviceptr wv, float a2) {
    void* a[] = {&v, &a1, &wv, &a2, &X, &Y, &Z};
    launch(k_ax, g1, 1, 1, 1024, 1, 1, a);
  };
  const auto t0 = std::chrono::steady_clock::now();
  for (uint32_t m = 0; m < n; ++m) {
    int i = (int)(m % wdt) - range, j = (int)((m / wdt) % wdt) - range, k = (int)(m / (wdt * wdt)) - range;
    void* ap[] = {&d_phi, &d_per, &X, &Y, &Z, &i, &j, &k, &dx, &dy, &dz, &kind, &ptype, &per, &px, &py, &pz,
                  &lcon, &lcon1, &sinez};
    launch(k_phi, g1, 1, 1, 1024, 1, 1, ap);
    if (!timing) w.arr(ddownload<float>(d_phi, P));
    // GPUCG_lattice(d_phi, iter, 1, EndRes, FinalIter, FinalRes)
    ck(cuMemcpyDtoD(d_d, d_phi, 4 * P), "cuMemcpyDtoD");
    ck(cuMemcpyDtoD(d_res, d_phi, 4 * P), "cuMemcpyDtoD");
    ck(cuMemsetD8(d_phi, 0, 4 * P), "cuMemsetD8");
    ck(cuMemsetD8(d_q, 0, 4 * P), "cuMemsetD8");
    (void)dot(d_res, d_res);
    float delta_new = dot(d_res, d_d);
    const float term = end_res * end_res;
    uint32_t it = 1;
    while (it < max_iter && delta_new > term) {
      void* am[] = {&d_d, &d_q, &X, &Y, &Z};
      launch(k_mv, g1, 1, 1, 1024, 1, 1, am);
      const float tmp = dot(d_d, d_q);
      const float alpha = delta_new / tmp;
      axpby(d_phi, 1.0f, d_d, alpha);
      axpby(d_res, 1.0f, d_q, (float)(-1.0 * alpha));
      const float delta_old = delta_new;
      delta_new = dot(d_res, d_res);
      const float beta = delta_new / delta_old;
      axpby(d_d, beta, d_res, 1.0f);
      ++it;
    }
    if (!timing) w.arr(ddownload<float>(d_phi, P));
    w.put<uint32_t>(it);
    CUDA_MEMCPY3D cp;
    std::memset(&cp, 0, sizeof(cp));
    cp.srcMemoryType = CU_MEMORYTYPE_DEVICE;
    cp.srcDevice = d_phi;
    cp.srcPitch = 4 * (size_t)X;
    cp.srcHeight = Y;
    cp.dstMemoryType = CU_MEMORYTYPE_ARRAY;
    cp.dstArray = arr;
    cp.WidthInBytes = 4 * (size_t)X;
    cp.Height = Y;
    cp.Depth = Z;
    ck(cuMemcpy3D(&cp), "cuMemcpy3D");
    int X2 = 2 * X, Y2 = 2 * Y, Z2 = 2 * Z;
    float dx2 = 0.5f * dx, dy2 = 0.5f * dy, dz2 = 0.5f * dz;
    void* ag[] = {&d_ga, &X2, &Y2, &Z2, &dx2, &dy2, &dz2, &tex};
    launch(k_gr, (unsigned)((X2 + 15) / 16), (unsigned)((Y2 + 15) / 16), (unsigned)((Z2 + 3) / 4), 16, 16, 4, ag);
    int mi = (int)m;
    void* as[] = {&d_svl, &d_ga, &X2, &Y2, &Z2, &mi, &d_coef};
    launch(k_svl, blocks_for(8 * P, 1024), 1, 1, 1024, 1, 1, as);
  }
  ck(cuCtxSynchronize(), "cuCtxSynchronize");
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (timing) w.put<double>(secs);
  else w.arr(ddownload<float>(d_svl, 8 * P));
  cuTexObjectDestroy(tex);
  cuArrayDestroy(arr);
  for (CUdeviceptr p : {d_phi, d_per, d_d, d_q, d_res, d_coef, d_svl, d_ga, d_red}) cuMemFree(p);
}

// kind 6: timing of the reference's plain marching-cubes kernels on one field.
// Per repetition classifyVoxel_new, compactVoxels and
// generateTriangles_lattice_kernel_3 are timed with events on a GB300, launched
// as the reference launches them (1024-thread classify and compaction, 32-thread
// generate, src/Isosurface.cu:44-150); the two scans run on the host between them
// and are not timed.  Writes nvox, active, total, reps, then per repetition the
// three kernel times (ms) and a checksum of the position words.
void run_mc_timing(Reader& r, Writer& w, CUmodule mc, const Tables& T) {
  U3 g{r.get<uint32_t>(), r.get<uint32_t>(), r.get<uint32_t>()};
  float iso = r.get<float>();
  F3 vs{r.get<float>(), r.get<float>(), r.get<float>()};
  F3 gc{r.get<float>(), r.get<float>(), r.get<float>()};
  uint32_t reps = r.get<uint32_t>();
  auto field = r.arr<float>((size_t)g.x * g.y * g.z);
  CUdeviceptr d_field = dupload(field);
  U3 mask{g.x - 1, g.y - 1, g.z - 1};
  U3 shift{1, g.x - 1, (g.x - 1) * (g.y - 1)};
  uint32_t nvox = mask.x * mask.y * mask.z;
  CUdeviceptr d_verts = dalloc<uint32_t>(nvox), d_occ = dalloc<uint32_t>(nvox);
  CUdeviceptr d_occ_scan = dalloc<uint32_t>(nvox), d_verts_scan = dalloc<uint32_t>(nvox);
  CUdeviceptr d_comp = dalloc<uint32_t>(nvox);
  CUfunction k_cls = find_kernel(mc, "classifyVoxel_new");
  CUfunction k_cmp = find_kernel(mc, "compactVoxels");
  CUfunction k_gen = find_kernel(mc, "generateTriangles_lattice_kernel_3");
  CUevent e0, e1;
  ck(cuEventCreate(&e0, CU_EVENT_DEFAULT), "cuEventCreate");
  ck(cuEventCreate(&e1, CU_EVENT_DEFAULT), "cuEventCreate");
  auto timed = [&](CUfunction f, unsigned gx, unsigned bx, void** a) {
    ck(cuEventRecord(e0, nullptr), "cuEventRecord");
    ck(cuLaunchKernel(f, gx, 1, 1, bx, 1, 1, 0, nullptr, a, nullptr), "cuLaunchKernel");
    ck(cuEventRecord(e1, nullptr), "cuEventRecord");
    ck(cuEventSynchronize(e1), "cuEventSynchronize");
    float ms = 0;
    ck(cuEventElapsedTime(&ms, e0, e1), "cuEventElapsedTime");
    return ms;
  };
  uint32_t active = 0, total = 0;
  CUdeviceptr d_pos = 0, d_norm = 0;
  uint32_t maxv = 0;
  std::vector<float> times;
  std::vector<uint64_t> sums;
  for (uint32_t rep = 0; rep < reps; ++rep) {
    void* ac[] = {&d_verts, &d_occ, &d_field, &g, &shift, &mask, &nvox, &vs, &iso,
                  const_cast<CUtexObject*>(&T.nverts_tex)};
    const float t_cls = timed(k_cls, blocks_for(nvox, 1024), 1024, ac);
    auto verts = ddownload<uint32_t>(d_verts, nvox);
    auto occ = ddownload<uint32_t>(d_occ, nvox);
    auto occ_scan = exclusive_scan(occ), verts_scan = exclusive_scan(verts);
    active = occ_scan.back() + occ.back();
    total = verts_scan.back() + verts.back();
    ck(cuMemcpyHtoD(d_occ_scan, occ_scan.data(), 4ull * nvox), "cuMemcpyHtoD");
    ck(cuMemcpyHtoD(d_verts_scan, verts_scan.data(), 4ull * nvox), "cuMemcpyHtoD");
    if (!d_pos) {
      maxv = total + 16;
      d_pos = dalloc<float>(4ull * maxv);
      d_norm = dalloc<float>(4ull * maxv);
    }
    void* am[] = {&d_comp, &d_occ, &d_occ_scan, &nvox};
    const float t_cmp = timed(k_cmp, blocks_for(nvox, 1024), 1024, am);
    void* ag[] = {&d_pos, &d_norm, &d_comp, &d_verts_scan, &g, &shift, &mask, &vs, &gc,
                  &iso, &active, &maxv, const_cast<CUtexObject*>(&T.tri_tex),
                  const_cast<CUtexObject*>(&T.nverts_tex), &total, &d_field, &iso};
    const float t_gen = active ? timed(k_gen, blocks_for(active, 32), 32, ag) : 0.0f;
    times.push_back(t_cls);
    times.push_back(t_cmp);
    times.push_back(t_gen);
    auto head = ddownload<uint32_t>(d_pos, 4ull * (total < 4096 ? total : 4096));
    uint64_t cs = 0;
    for (uint32_t v : head) cs = cs * 1000003ull + v;
    sums.push_back(cs);
  }
  w.put<uint32_t>(nvox);
  w.put<uint32_t>(active);
  w.put<uint32_t>(total);
  w.put<uint32_t>(reps);
  w.arr(times);
  w.arr(sums);
  cuEventDestroy(e0); cuEventDestroy(e1);
  cuMemFree(d_field); cuMemFree(d_verts); cuMemFree(d_occ); cuMemFree(d_occ_scan);
  cuMemFree(d_verts_scan); cuMemFree(d_comp);
  if (d_pos) { cuMemFree(d_pos); cuMemFree(d_norm); }
}

int main(int argc, char** argv) {
  if (argc != 6) {
    std::fprintf(stderr, "usage: ref_runner <fatbin-dir> <sm103a|ptx89> <tables.bin> <job.bin> <out.bin>\n");
    return 2;
  }
  std::string dir = argv[1], var = argv[2];
  ck(cuInit(0), "cuInit");
  CUdevice dev;
  ck(cuDeviceGet(&dev, 0), "cuDeviceGet");
  CUcontext ctx;
  CUctxCreateParams cp;
  std::memset(&cp, 0, sizeof(cp));
  ck(cuCtxCreate(&ctx, &cp, 0, dev), "cuCtxCreate");
  auto load = [&](const char* unit) {
    auto img = slurp(dir + "/ref_" + unit + "_" + var + ".fatbin");
    CUmodule m;
    ck(cuModuleLoadData(&m, img.data()), "cuModuleLoadData");
    return m;
  };
  CUmodule mc = load("mc"), mdl = load("modelling"), fft = load("fft"), gr = load("gratings");
  Tables T = load_tables(argv[3]);
  auto job = slurp(argv[4]);
  Reader r{job};
  FILE* of = std::fopen(argv[5], "wb");
  if (!of) die("cannot open output");
  Writer w{of};
  if (r.get<uint32_t>() != 0x4A4D4347u) die("bad job magic");
  uint32_t ncases = r.get<uint32_t>();
  for (uint32_t i = 0; i < ncases; ++i) {
    uint32_t kind = r.get<uint32_t>();
    w.put<uint32_t>(kind);
    switch (kind) {
      case 1: run_mc_plain(r, w, mc, T); break;
      case 2: run_mc_band(r, w, mc, T); break;
      case 3: run_unit_cell(r, w, fft); break;
      case 4: run_primitive(r, w, mdl); break;
      case 5: run_normalise_four(r, w, gr); break;
      case 6: run_mc_timing(r, w, mc, T); break;
      case 7: run_retain(r, w, mc, T, false); break;
      case 10: run_retain(r, w, mc, T, true); break;
      case 8: run_svl(r, w, gr, false); break;
      case 9: run_svl(r, w, gr, true); break;
      case 11: run_period(r, w, gr); break;
      case 12: run_mask(r, w, gr); break;
      default: die("unknown job kind");
    }
  }
  std::fclose(of);
  cuCtxDestroy(ctx);
  std::printf("ref_runner: %u cases done (%s)\n", ncases, var.c_str());
  return 0;
}
