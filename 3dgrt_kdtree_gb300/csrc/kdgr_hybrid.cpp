// kdgr_hybrid.cpp -- the secondary-ray hybrid render path: Gaussians plus
// mirror/glass/opaque secondary primitives (spheres, a triangle mesh), the
// reference's SECONDARY_RAY build of the renderer (renderKernelGaussian_Mesh_
// Hybrid, cudaRenderer.cu:2217-2311; SecondaryMesh, cudaRenderer.h:12-29;
// loadSecondaryMesh, Kd-treeConverterMain.cpp:179-221).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "kdgr.h"
#include "kdgr_internal.h"
#include "scene.h"

using namespace kdgr;

struct kdgr_secondary_s {
  float* d_spheres = nullptr;
  float* d_tris = nullptr;
  float* d_tri_material = nullptr;
  int n_spheres = 0;
  uint32_t n_tris = 0;
};

namespace {

void material_words(const kdgr_material& m, float out[6]) {
  memcpy(&out[0], &m.material, 4);
  out[1] = m.reflectivity;
  out[2] = m.ior;
  out[3] = m.color[0];
  out[4] = m.color[1];
  out[5] = m.color[2];
}

bool material_ok(const kdgr_material& m) { return m.material >= 0 && m.material <= 2; }

// Parse one OBJ face-vertex token ("v", "v/vt", "v//vn", "v/vt/vn") into a
// zero-based position index; negative indices count from the end.
bool obj_index(const char* tok, long n_pos, long* out) {
  char* end = nullptr;
  const long i = strtol(tok, &end, 10);
  if (end == tok || i == 0) return false;
  const long k = i > 0 ? i - 1 : n_pos + i;
  if (k < 0 || k >= n_pos) return false;
  *out = k;
  return true;
}

}  // namespace

extern "C" {

int kdgr_demo_spheres(kdgr_sphere out[2]) {
  if (!out) {
    set_error("kdgr_demo_spheres: null output");
    return KDGR_ERR_INVALID_ARG;
  }
  // demo_spheres (cudaRenderer.cu:2158-2168): a glass sphere (ior 1.1) and a mirror
  out[0] = kdgr_sphere{{0.0f, 1.0f, 0.0f}, 0.3f, {2, 1.0f, 1.1f, {1.0f, 1.0f, 1.0f}}};
  out[1] = kdgr_sphere{{0.8f, 1.0f, 1.2f}, 0.3f, {1, 1.0f, 1.0f, {1.0f, 1.0f, 1.0f}}};
  return KDGR_OK;
}

void kdgr_secondary_mesh_material_default(kdgr_material* m) {
  if (!m) return;
  // SecondaryMesh defaults (cudaRenderer.h:12-19) with materialType 1 as the
  // caller sets it (Kd-treeConverterMain.cpp:3054)
  *m = kdgr_material{1, 0.95f, 1.1f, {0.95f, 0.95f, 0.95f}};
}

int kdgr_read_obj(const char* path, float** verts, uint32_t* n_tris) {
  if (!path || !verts || !n_tris) {
    set_error("kdgr_read_obj: null argument");
    return KDGR_ERR_INVALID_ARG;
  }
  *verts = nullptr;
  *n_tris = 0;
  FILE* fp = fopen(path, "r");
  if (!fp) {
    set_error(std::string("kdgr_read_obj: cannot open ") + path);
    return KDGR_ERR_IO;
  }
  std::vector<float> pos, tri;
  char line[4096];
  int line_no = 0;
  while (fgets(line, sizeof line, fp)) {
    ++line_no;
    const char* p = line;
    while (*p == ' ' || *p == '\t') ++p;
    if (p[0] == 'v' && (p[1] == ' ' || p[1] == '\t')) {
      float x, y, z;
      if (sscanf(p + 2, "%f %f %f", &x, &y, &z) != 3) {
        fclose(fp);
        set_error("kdgr_read_obj: bad vertex on line " + std::to_string(line_no));
        return KDGR_ERR_FORMAT;
      }
      pos.insert(pos.end(), {x, y, z});
    } else if (p[0] == 'f' && (p[1] == ' ' || p[1] == '\t')) {
      std::vector<long> idx;
      char* save = nullptr;
      std::string rest(p + 2);
      for (char* tok = strtok_r(&rest[0], " \t\r\n", &save); tok; tok = strtok_r(nullptr, " \t\r\n", &save)) {
        long k;
        if (!obj_index(tok, (long)(pos.size() / 3), &k)) {
          fclose(fp);
          set_error("kdgr_read_obj: bad face index on line " + std::to_string(line_no));
          return KDGR_ERR_FORMAT;
        }
        idx.push_back(k);
      }
      if (idx.size() < 3) {
        fclose(fp);
        set_error("kdgr_read_obj: face with fewer than 3 vertices on line " + std::to_string(line_no));
        return KDGR_ERR_FORMAT;
      }
      // fan triangulation (the loader triangulates polygons), then the
      // reference's axis change: (x, y, z) -> (x, -z, y)
      for (size_t k = 1; k + 1 < idx.size(); ++k)
        for (long v : {idx[0], idx[k], idx[k + 1]})
          tri.insert(tri.end(), {pos[3 * v], -pos[3 * v + 2], pos[3 * v + 1]});
    }
  }
  fclose(fp);
  if (tri.empty()) {
    set_error("kdgr_read_obj: no faces");
    return KDGR_ERR_FORMAT;
  }
  *verts = (float*)malloc(tri.size() * sizeof(float));
  if (!*verts) {
    set_error("kdgr_read_obj: host allocation failed");
    return KDGR_ERR_OUT_OF_MEMORY;
  }
  memcpy(*verts, tri.data(), tri.size() * sizeof(float));
  *n_tris = (uint32_t)(tri.size() / 9);
  return KDGR_OK;
}

void kdgr_free(void* p) { free(p); }

int kdgr_secondary_create(const kdgr_sphere* spheres, int n_spheres, const float* tri_verts, uint32_t n_tris,
                          const kdgr_material* tri_material, kdgr_secondary_t* out) {
  if (!out || n_spheres < 0 || (n_spheres > 0 && !spheres) || (n_tris > 0 && (!tri_verts || !tri_material))) {
    set_error("kdgr_secondary_create: null argument or negative count");
    return KDGR_ERR_INVALID_ARG;
  }
  if (n_spheres > 4096) {
    set_error("kdgr_secondary_create: at most 4096 spheres");
    return KDGR_ERR_LIMIT;
  }
  std::vector<float> sph(10 * (size_t)n_spheres);
  for (int i = 0; i < n_spheres; ++i) {
    const kdgr_sphere& s = spheres[i];
    if (!material_ok(s.material) || !(s.radius > 0.f)) {
      set_error("kdgr_secondary_create: sphere " + std::to_string(i) + " has a bad radius or material");
      return KDGR_ERR_INVALID_ARG;
    }
    memcpy(&sph[10 * i], s.center, 12);
    sph[10 * i + 3] = s.radius;
    material_words(s.material, &sph[10 * i + 4]);
  }
  float tm[6] = {0, 0, 0, 0, 0, 0};
  if (n_tris > 0) {
    if (!material_ok(*tri_material)) {
      set_error("kdgr_secondary_create: bad mesh material");
      return KDGR_ERR_INVALID_ARG;
    }
    material_words(*tri_material, tm);
  }
  kdgr_secondary_s* s = new kdgr_secondary_s;
  s->n_spheres = n_spheres;
  s->n_tris = n_tris;
  cudaError_t e = cudaSuccess;
  if (n_spheres > 0) {
    e = cudaMalloc(&s->d_spheres, sph.size() * 4);
    if (e == cudaSuccess) e = cudaMemcpy(s->d_spheres, sph.data(), sph.size() * 4, cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess && n_tris > 0) {
    e = cudaMalloc(&s->d_tris, 36ull * n_tris);
    if (e == cudaSuccess) e = cudaMemcpy(s->d_tris, tri_verts, 36ull * n_tris, cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess) e = cudaMalloc(&s->d_tri_material, sizeof tm);
  if (e == cudaSuccess) e = cudaMemcpy(s->d_tri_material, tm, sizeof tm, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(s->d_spheres);
    cudaFree(s->d_tris);
    cudaFree(s->d_tri_material);
    delete s;
    return cuda_fail(e, "kdgr_secondary_create");
  }
  *out = s;
  return KDGR_OK;
}

int kdgr_secondary_destroy(kdgr_secondary_t s) {
  if (!s) return KDGR_OK;
  cudaFree(s->d_spheres);
  cudaFree(s->d_tris);
  cudaFree(s->d_tri_material);
  delete s;
  return KDGR_OK;
}

int kdgr_render_hybrid(kdgr_scene_t s, const kdgr_camera* cam, int W, int H, kdgr_secondary_t sec, float* rgb,
                       void* stream, float* ms_out) {
  if (!s || !cam || !sec || !rgb || W <= 0 || H <= 0) {
    set_error("kdgr_render_hybrid: null scene/camera/secondary/output or empty image");
    return KDGR_ERR_INVALID_ARG;
  }
  if (!(s->forms & KDGR_FORM_EXACT)) {
    set_error("kdgr_render_hybrid: scene was created without KDGR_FORM_EXACT");
    return KDGR_ERR_INVALID_ARG;
  }
  DeviceScope on(s->device);
  if (on.err != cudaSuccess) return cuda_fail(on.err, "kdgr_render_hybrid");
  const cudaStream_t st = (cudaStream_t)stream;
  const CamInfo ci = make_caminfo(*cam, W, H);
  HybridView m{sec->d_spheres, sec->d_tris, sec->d_tri_material, sec->n_spheres, sec->n_tris};
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (ms_out) {
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
  }
  cudaError_t e = launch_hybrid(s->exact_view(), ci, W, H, m, rgb, s->d_status, st);
  if (e == cudaSuccess && ms_out) {
    cudaEventRecord(e1, st);
    e = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    *ms_out = ms;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (e != cudaSuccess) return cuda_fail(e, "kdgr_render_hybrid");
  return KDGR_OK;
}

}  // extern "C"
