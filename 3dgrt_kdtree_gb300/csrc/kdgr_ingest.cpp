// kdgr_ingest.cpp -- Gaussian scene ingest from 3D Gaussian Splatting `.ply`
// files: loadGaussiansFromPly (Kd-treeConverterMain.cpp:1652-1769) as a
// library call.
//
// The header is read line by line up to `end_header`; the vertex element's
// properties give each field's byte offset within a vertex; the binary
// little-endian vertex block is then read in one piece and activated in
// parallel into the reference's 64-float Gaussian records:
//   pos      = x, y, z
//   opacity  = 1 / (1 + exp(-opacity))             (:1729)
//   scale[i] = exp(scale_i)                        (:1731-1734)
//   rot      = rot_0..3 normalised when |q|^2 > 1e-5 (fMyVecNormalize4D :1568-1577, :1737-1738)
//   k_scale  = calcKernelScale(opacity)            (Gaussian.h:6-15, :1747)
//   f_dc     = f_dc_0..2, f_rest = f_rest_0..44 (zero when absent)
// exp is evaluated in double and rounded once to float: the correctly
// rounded float result in all but vanishingly rare cases, which is what an
// accurate host expf returns.
//
// Differences from the reference loader, all on malformed or unusual files
// (it reads them wrongly or not at all): the `format` line must say
// binary_little_endian; every PLY scalar type has its size (the reference
// sizes float/double/uchar only); properties of elements other than `vertex`
// do not shift the vertex offsets; each required field is looked up by its
// own name and must be a float; a short read is an error.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "kdgr.h"
#include "kdgr_internal.h"
#include "scene.h"

namespace kdgr {
namespace {

struct PlyProp {
  int offset;
  int size;
  bool is_float;
};

int type_size(const std::string& t, bool* is_float) {
  *is_float = (t == "float" || t == "float32");
  if (t == "char" || t == "uchar" || t == "int8" || t == "uint8") return 1;
  if (t == "short" || t == "ushort" || t == "int16" || t == "uint16") return 2;
  if (t == "int" || t == "uint" || t == "int32" || t == "uint32" || *is_float) return 4;
  if (t == "double" || t == "float64") return 8;
  return 0;
}

inline float exp_f(float x) { return (float)std::exp((double)x); }

// calcKernelScale (Gaussian.h:6-15) with ADAPTIVE_KERNEL_CLAMPING and
// KERNEL_DEGREE 4: the radius where the kernel falls to the clamped minimum
// response.  Not read by the render path; filled so records match.
inline float kernel_scale(float density) {
  const float min_resp = std::min(0.0113f / density, 0.97f);
  const float a = -4.5f / 81.0f;  // -4.5 / 3^KERNEL_DEGREE
  const float l = (float)std::log((double)min_resp);
  return (float)std::pow((double)(l / a), 0.25);  // 1 / KERNEL_DEGREE
}

void activate(const uint8_t* v, const int off[16], float* r) {
  auto f = [&](int o) {
    float x;
    memcpy(&x, v + o, 4);
    return x;
  };
  for (int i = 0; i < 64; ++i) r[i] = 0.f;
  r[0] = f(off[0]);
  r[1] = f(off[1]);
  r[2] = f(off[2]);
  const float op = 1.0f / (1.0f + exp_f(-f(off[3])));
  r[3] = op;
  for (int i = 0; i < 3; ++i) r[4 + i] = exp_f(f(off[4 + i]));
  float q[4] = {f(off[7]), f(off[8]), f(off[9]), f(off[10])};
  const float len_sq = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
  if (len_sq > 0.00001f) {
    const float inv = 1.0f / std::sqrt(len_sq);
    for (int i = 0; i < 4; ++i) q[i] *= inv;
  }
  for (int i = 0; i < 4; ++i) r[8 + i] = q[i];
  r[7] = kernel_scale(op);
  for (int i = 0; i < 3; ++i) r[12 + i] = f(off[11 + i]);
  if (off[14] >= 0)
    for (int i = 0; i < 45; ++i) r[15 + i] = f(off[14] + 4 * i);
}

}  // namespace

int parse_ply_header(FILE* fp, PlyLayout& lay, uint64_t& n_out, uint32_t& stride_out, std::string& err) {
  auto fail = [&](const std::string& m, int code) {
    err = m;
    return code;
  };
  char buf[4096];
  if (!fgets(buf, sizeof buf, fp) || strncmp(buf, "ply", 3) != 0) return fail("not a PLY file", KDGR_ERR_FORMAT);
  std::map<std::string, PlyProp> props;
  std::string current;
  long long n_vertices = -1;
  int stride = 0;
  bool little = false, done = false;
  while (fgets(buf, sizeof buf, fp)) {
    std::string line(buf);
    while (!line.empty() && (line.back() == '\n' || line.back() == '\r')) line.pop_back();
    if (line == "end_header") {
      done = true;
      break;
    }
    std::stringstream ss(line);
    std::string tok;
    ss >> tok;
    if (tok == "format") {
      std::string f;
      ss >> f;
      little = (f == "binary_little_endian");
    } else if (tok == "element") {
      long long cnt = -1;
      ss >> current >> cnt;
      if (current == "vertex") {
        if (n_vertices >= 0) return fail("two vertex elements", KDGR_ERR_FORMAT);
        n_vertices = cnt;
      } else if (n_vertices < 0) {
        return fail("element '" + current + "' before the vertex element", KDGR_ERR_FORMAT);
      }
    } else if (tok == "property" && current == "vertex") {
      std::string type, name;
      ss >> type;
      if (type == "list") return fail("list property in the vertex element", KDGR_ERR_FORMAT);
      ss >> name;
      bool is_float = false;
      const int sz = type_size(type, &is_float);
      if (sz == 0) return fail("unknown PLY type '" + type + "'", KDGR_ERR_FORMAT);
      props[name] = {stride, sz, is_float};
      stride += sz;
    }
  }
  if (!done) return fail("no end_header", KDGR_ERR_FORMAT);
  if (!little) return fail("only binary_little_endian PLY is supported", KDGR_ERR_FORMAT);
  if (n_vertices <= 0) return fail("no vertices", KDGR_ERR_FORMAT);
  if (n_vertices > 0xFFFFFFFFll) return fail("more than 2^32-1 vertices", KDGR_ERR_LIMIT);

  static const char* kNeed[14] = {"x",       "y",       "z",       "opacity", "scale_0", "scale_1", "scale_2",
                                  "rot_0",   "rot_1",   "rot_2",   "rot_3",   "f_dc_0",  "f_dc_1",  "f_dc_2"};
  for (int i = 0; i < 14; ++i) {
    auto it = props.find(kNeed[i]);
    if (it == props.end() || !it->second.is_float)
      return fail(std::string("missing float property '") + kNeed[i] + "'", KDGR_ERR_FORMAT);
    lay.off[i] = it->second.offset;
  }
  lay.off[14] = -1;
  lay.off[15] = 0;
  auto r0 = props.find("f_rest_0");
  if (r0 != props.end()) {
    for (int k = 0; k < 45; ++k) {
      auto it = props.find("f_rest_" + std::to_string(k));
      if (it == props.end() || !it->second.is_float || it->second.offset != r0->second.offset + 4 * k)
        return fail("f_rest_0..44 must be 45 consecutive floats", KDGR_ERR_FORMAT);
    }
    lay.off[14] = r0->second.offset;
  }
  n_out = (uint64_t)n_vertices;
  stride_out = (uint32_t)stride;
  return KDGR_OK;
}

namespace {

int read_ply(const char* path, std::vector<float>& rec, uint32_t& n_out, std::string& err) {
  FILE* fp = fopen(path, "rb");
  if (!fp) {
    err = std::string("cannot open ") + path;
    return KDGR_ERR_IO;
  }
  PlyLayout lay;
  uint64_t n_vertices = 0;
  uint32_t stride = 0;
  int rc = parse_ply_header(fp, lay, n_vertices, stride, err);
  if (rc != KDGR_OK) {
    fclose(fp);
    return rc;
  }
  const size_t n = (size_t)n_vertices;
  std::vector<uint8_t> raw;
  try {
    raw.resize(n * (size_t)stride);
    rec.assign(n * 64, 0.f);
  } catch (const std::bad_alloc&) {
    fclose(fp);
    err = "host allocation failed for " + std::to_string(n) + " vertices";
    return KDGR_ERR_OUT_OF_MEMORY;
  }
  if (fread(raw.data(), 1, raw.size(), fp) != raw.size()) {
    fclose(fp);
    err = "vertex data shorter than the header announces";
    return KDGR_ERR_FORMAT;
  }
  fclose(fp);

  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const size_t per = std::max<size_t>(16384, (n + hw - 1) / hw);
  std::vector<std::thread> pool;
  for (size_t b = 0; b < n; b += per) {
    const size_t e = std::min(n, b + per);
    pool.emplace_back([&, b, e] {
      for (size_t i = b; i < e; ++i) activate(raw.data() + i * stride, lay.off, rec.data() + 64 * i);
    });
  }
  for (auto& t : pool) t.join();
  n_out = (uint32_t)n;
  return KDGR_OK;
}

}  // namespace
}  // namespace kdgr

using namespace kdgr;

extern "C" int kdgr_read_ply(const char* path, kdgr_gaussians* out) {
  if (!path || !out) {
    set_error("kdgr_read_ply: null argument");
    return KDGR_ERR_INVALID_ARG;
  }
  memset(out, 0, sizeof *out);
  std::vector<float> rec;
  uint32_t n = 0;
  std::string err;
  const int rc = read_ply(path, rec, n, err);
  if (rc != KDGR_OK) {
    set_error("kdgr_read_ply: " + err);
    return rc;
  }
  out->records = (float*)malloc(rec.size() * sizeof(float));
  if (!out->records) {
    set_error("kdgr_read_ply: host allocation failed");
    return KDGR_ERR_OUT_OF_MEMORY;
  }
  memcpy(out->records, rec.data(), rec.size() * sizeof(float));
  out->n = n;
  return KDGR_OK;
}

extern "C" void kdgr_gaussians_free(kdgr_gaussians* g) {
  if (!g) return;
  free(g->records);
  g->records = nullptr;
  g->n = 0;
}

namespace kdgr {
namespace {

// Stream the PLY vertex block to the device in chunks through two pinned
// buffers, activating each chunk on the device while the next is read.
int read_ply_device(const char* path, float* d_rec, uint32_t capacity, uint32_t* n_out, cudaStream_t st,
                    std::string& err) {
  FILE* fp = fopen(path, "rb");
  if (!fp) {
    err = std::string("cannot open ") + path;
    return KDGR_ERR_IO;
  }
  PlyLayout lay;
  uint64_t n = 0;
  uint32_t stride = 0;
  int rc = parse_ply_header(fp, lay, n, stride, err);
  if (rc != KDGR_OK || !d_rec) {
    fclose(fp);
    if (rc == KDGR_OK) *n_out = (uint32_t)n;
    return rc;
  }
  if (n > capacity) {
    fclose(fp);
    err = std::to_string(n) + " vertices exceed the capacity of " + std::to_string(capacity) + " records";
    return KDGR_ERR_LIMIT;
  }
  const uint64_t per = std::max<uint64_t>(1, (16ull << 20) / stride);  // vertices per chunk (about 16 MB)
  const size_t bytes = (size_t)per * stride;
  uint8_t* host[2] = {nullptr, nullptr};
  uint8_t* dev[2] = {nullptr, nullptr};
  cudaEvent_t ev[2] = {nullptr, nullptr};
  cudaError_t e = cudaSuccess;
  for (int b = 0; b < 2 && e == cudaSuccess; ++b) {
    e = cudaMallocHost(&host[b], bytes);
    if (e == cudaSuccess) e = cudaMalloc(&dev[b], bytes);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev[b], cudaEventDisableTiming);
  }
  uint64_t first = 0;
  for (uint64_t c = 0; e == cudaSuccess && first < n; ++c) {
    const int b = (int)(c & 1);
    const uint64_t nv = std::min(per, n - first);
    if (c >= 2) e = cudaEventSynchronize(ev[b]);  // the copy out of host[b] two chunks ago is done
    if (e != cudaSuccess) break;
    if (fread(host[b], 1, (size_t)nv * stride, fp) != (size_t)nv * stride) {
      rc = KDGR_ERR_FORMAT;
      err = "vertex data shorter than the header announces";
      break;
    }
    e = cudaMemcpyAsync(dev[b], host[b], (size_t)nv * stride, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaEventRecord(ev[b], st);
    if (e == cudaSuccess) e = launch_ply_activate(dev[b], (uint32_t)nv, stride, lay, d_rec + 64ull * first, st);
    first += nv;
  }
  const cudaError_t es = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = es;
  for (int b = 0; b < 2; ++b) {
    if (host[b]) cudaFreeHost(host[b]);
    if (dev[b]) cudaFree(dev[b]);
    if (ev[b]) cudaEventDestroy(ev[b]);
  }
  fclose(fp);
  if (rc != KDGR_OK) return rc;
  if (e != cudaSuccess) {
    err = std::string("CUDA: ") + cudaGetErrorString(e);
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? KDGR_ERR_OUT_OF_MEMORY : KDGR_ERR_CUDA;
  }
  *n_out = (uint32_t)n;
  return KDGR_OK;
}

}  // namespace
}  // namespace kdgr

extern "C" int kdgr_read_ply_device(const char* path, float* d_records, uint32_t capacity, uint32_t* n_out,
                                    void* stream) {
  if (!path || !n_out) {
    set_error("kdgr_read_ply_device: null argument");
    return KDGR_ERR_INVALID_ARG;
  }
  std::string err;
  const int rc = read_ply_device(path, d_records, capacity, n_out, (cudaStream_t)stream, err);
  if (rc != KDGR_OK) set_error("kdgr_read_ply_device: " + err);
  return rc;
}

extern "C" int kdgr_scene_create_from_files(const char* ply_path, const char* kdt_path, uint32_t flags,
                                            kdgr_scene_t* out) {
  if (!ply_path || !kdt_path || !out) {
    set_error("kdgr_scene_create_from_files: null argument");
    return KDGR_ERR_INVALID_ARG;
  }
  if (flags & KDGR_SCALES_INVERTED) {
    set_error("kdgr_scene_create_from_files: PLY records are activated, not inverted (drop KDGR_SCALES_INVERTED)");
    return KDGR_ERR_INVALID_ARG;
  }
  *out = nullptr;
  std::string err;
  HostTree t;
  int rc = read_kdt(kdt_path, t, err);
  if (rc != KDGR_OK) {
    set_error("kdgr_scene_create_from_files: " + err);
    return rc;
  }
  uint32_t n = 0;
  rc = read_ply_device(ply_path, nullptr, 0, &n, nullptr, err);  // vertex count from the header
  if (rc != KDGR_OK) {
    set_error("kdgr_scene_create_from_files: " + err);
    return rc;
  }
  const uint32_t n_nodes = (uint32_t)(t.nodes.size() / 2), n_offsets = (uint32_t)t.offsets.size();
  uint32_t depth = 0;
  rc = validate_tree(t.nodes.data(), n_nodes, t.offsets.data(), n_offsets, n, err, &depth);
  if (rc != KDGR_OK) {
    set_error("kdgr_scene_create_from_files: " + err);
    return rc;
  }
  float* d_rec = nullptr;
  cudaError_t e = cudaMalloc(&d_rec, 256ull * n);
  if (e != cudaSuccess) return cuda_fail(e, "kdgr_scene_create_from_files: cudaMalloc");
  uint32_t n2 = 0;
  rc = read_ply_device(ply_path, d_rec, n, &n2, nullptr, err);
  if (rc != KDGR_OK) {
    cudaFree(d_rec);
    set_error("kdgr_scene_create_from_files: " + err);
    return rc;
  }
  rc = scene_create_impl(t.nodes.data(), n_nodes, t.offsets.data(), n_offsets, t.aabb, d_rec, n, flags, depth, out,
                         "kdgr_scene_create_from_files");
  cudaFree(d_rec);
  return rc;
}
