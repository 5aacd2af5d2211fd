// kdgr_reference_api.cpp -- the reference's C++ render entry points
// (include/kdgr_reference_api.h) over the C ABI.  One global scene and the
// last frame's parameters, as the reference keeps global device state
// (cudaRenderer.cu:314-360).
#include "kdgr_reference_api.h"

#include <algorithm>
#include <cstdio>
#include <string>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "kdgr.h"

namespace {

std::mutex g_mu;
kdgr_scene_t g_scene = nullptr;
kdgr_tree g_tree;  // arrays handed out by read_kd_tree_from_file
bool g_have_tree = false;
bool g_have_frame = false;
kdgr_camera g_last_cam;
int g_last_w = 0, g_last_h = 0;
// SECONDARY_RAY build: secondary primitives (demo spheres and/or mesh)
kdgr_secondary_t g_sec_spheres = nullptr, g_sec_mesh = nullptr;
bool g_hybrid = false;
int g_secondary_prim = KDGR_SECONDARY_SPHERE;

void drop_secondary() {
  if (g_sec_spheres) kdgr_secondary_destroy(g_sec_spheres);
  if (g_sec_mesh) kdgr_secondary_destroy(g_sec_mesh);
  g_sec_spheres = g_sec_mesh = nullptr;
  g_hybrid = false;
}

std::string g_debug_dir;  // non-empty: per-frame HIT_AND_NODE_COUNT_DEBUG report

// Trace the frame with the oracle-matching kernel and write the report.
int debug_report_frame(const kdgr_camera& cam, int width, int height, cudaStream_t stream) {
  const size_t n = (size_t)width * height;
  kdgr_ray_trace* d_tr = nullptr;
  float* d_rgb = nullptr;
  cudaError_t e = cudaMalloc(&d_tr, n * sizeof(kdgr_ray_trace));
  if (e == cudaSuccess) e = cudaMalloc(&d_rgb, n * 3 * sizeof(float));
  int rc = e == cudaSuccess ? KDGR_OK : KDGR_ERR_OUT_OF_MEMORY;
  std::vector<kdgr_ray_trace> h(n);
  if (rc == KDGR_OK) rc = kdgr_render_trace(g_scene, &cam, width, height, d_rgb, nullptr, nullptr, d_tr, (void*)stream);
  if (rc == KDGR_OK && cudaStreamSynchronize(stream) != cudaSuccess) rc = KDGR_ERR_CUDA;
  if (rc == KDGR_OK && cudaMemcpy(h.data(), d_tr, n * sizeof(kdgr_ray_trace), cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = KDGR_ERR_CUDA;
  cudaFree(d_tr);
  cudaFree(d_rgb);
  kdgr_debug_stats st;
  if (rc == KDGR_OK) rc = kdgr_debug_report(h.data(), width, height, g_debug_dir.c_str(), 120.0f, &st);
  if (rc == KDGR_OK) {
    printf("\n===========================================\n");
    printf("avg_node_visits\t\t: %f\n", (double)st.avg[0]);
    printf("avg_intersection_tests\t: %f\n", (double)st.avg[2]);
    printf("avg_blend_ops\t\t: %f\n", (double)st.avg[4]);
    printf("===========================================\n");
  }
  return rc;
}

int render_frame(const kdgr_camera& cam, int width, int height, float* fb, cudaStream_t stream, float* ms) {
  if (!g_debug_dir.empty() && debug_report_frame(cam, width, height, stream) != KDGR_OK)
    fprintf(stderr, "[CUDA Error] debug report failed: %s\n", kdgr_last_error());
  if (g_hybrid) {
    kdgr_secondary_t sec = g_secondary_prim == KDGR_SECONDARY_TRI ? g_sec_mesh : g_sec_spheres;
    return kdgr_render_hybrid(g_scene, &cam, width, height, sec, fb, (void*)stream, ms);
  }
  return kdgr_render(g_scene, &cam, width, height, fb, nullptr, nullptr, (void*)stream, ms);
}

kdgr_camera to_camera(const Camera& c) {
  kdgr_camera k;
  for (int i = 0; i < 3; ++i) {
    k.pos[i] = c.pos[i];
    k.uaxis[i] = c.uaxis[i];
    k.vaxis[i] = c.vaxis[i];
    k.naxis[i] = c.naxis[i];
  }
  k.fovy = c.fovy;
  k.aspect = c.aspect;
  k.near_c = c.near_c;
  return k;
}

}  // namespace

bool initCuda() {
  const int rc = kdgr_init(0);
  if (rc != KDGR_OK) {
    fprintf(stderr, "[CUDA Init] %s\n", kdgr_last_error());
    return false;
  }
  return true;
}

void renderGaussianWithCudaSetup(const CompositeObject& object, const std::vector<Gaussian>& gaussians) {
  static_assert(sizeof(Gaussian) == 256, "Gaussian must be the reference's 256-byte record");
  std::lock_guard<std::mutex> lk(g_mu);
  const KdTree* t = object.kd_tree;
  if (!t || gaussians.empty()) {
    fprintf(stderr, "[CUDA Error] Kd-tree or Gaussian data is empty.\n");
    return;
  }
  if (g_scene) {
    kdgr_scene_destroy(g_scene);
    g_scene = nullptr;
  }
  drop_secondary();
  if (const char* dd = getenv("KDGR_DEBUG_REPORT_DIR")) g_debug_dir = dd;
  // CompositeObject.AABB is (xmin, xmax, ymin, ymax, zmin, zmax); the scene
  // takes the .kdt order (xmin, ymin, zmin, xmax, ymax, zmax)
  const float aabb[6] = {object.AABB[0], object.AABB[2], object.AABB[4],
                         object.AABB[1], object.AABB[3], object.AABB[5]};
  const int rc = kdgr_scene_create(reinterpret_cast<const uint32_t*>(t->tree), (uint32_t)t->tree_node_count,
                                   t->prim_offset_list, (uint32_t)t->prim_offset_count, aabb,
                                   reinterpret_cast<const float*>(gaussians.data()), (uint32_t)gaussians.size(),
                                   KDGR_SCALES_INVERTED | KDGR_FORM_EXACT, &g_scene);
  if (rc != KDGR_OK) {
    fprintf(stderr, "[CUDA Error] setup failed: %s\n", kdgr_last_error());
    g_scene = nullptr;
  }
}

void renderGaussianWithCudaSetup(const CompositeObject& object, const std::vector<Gaussian>& gaussians,
                                 SecondaryMesh& secondaryMesh) {
  renderGaussianWithCudaSetup(object, gaussians);
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scene) return;
  kdgr_sphere sph[2];
  kdgr_demo_spheres(sph);
  int rc = kdgr_secondary_create(sph, 2, nullptr, 0, nullptr, &g_sec_spheres);
  const uint32_t n_tris = (uint32_t)std::min<size_t>((size_t)std::max(secondaryMesh.triangleCount, 0),
                                                     secondaryMesh.vert.size() / 3);
  kdgr_material mat{secondaryMesh.materialType, secondaryMesh.reflectivity, secondaryMesh.ior,
                    {secondaryMesh.color.x, secondaryMesh.color.y, secondaryMesh.color.z}};
  if (rc == KDGR_OK)
    rc = kdgr_secondary_create(nullptr, 0, reinterpret_cast<const float*>(secondaryMesh.vert.data()), n_tris, &mat,
                               &g_sec_mesh);
  if (rc != KDGR_OK) {
    fprintf(stderr, "[CUDA Error] secondary mesh setup failed: %s\n", kdgr_last_error());
    drop_secondary();
    return;
  }
  g_hybrid = true;
}

void setDebugReportDir(const char* dir) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_debug_dir = dir ? dir : "";
}

void setSecondaryPrimitive(int prim) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_secondary_prim = prim == KDGR_SECONDARY_TRI ? KDGR_SECONDARY_TRI : KDGR_SECONDARY_SPHERE;
}

float renderGaussianWithCudaFrame(const Camera& camera, int width, int height, float* d_framebuffer,
                                  cudaStream_t stream) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scene) {
    fprintf(stderr, "[CUDA Error] renderGaussianWithCudaFrame before renderGaussianWithCudaSetup\n");
    return 0.f;
  }
  const kdgr_camera cam = to_camera(camera);
  float ms = 0.f;
  const int rc = render_frame(cam, width, height, d_framebuffer, stream, &ms);
  if (rc != KDGR_OK) {
    fprintf(stderr, "[CUDA Error] render failed: %s\n", kdgr_last_error());
    return 0.f;
  }
  g_last_cam = cam;
  g_last_w = width;
  g_last_h = height;
  g_have_frame = true;
  return ms > 0.f ? 1000.0f / ms : 0.f;
}

void warmUp(float* d_framebuffer, cudaStream_t stream) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scene || !g_have_frame) return;
  float ms = 0.f;
  if (render_frame(g_last_cam, g_last_w, g_last_h, d_framebuffer, stream, &ms) == KDGR_OK)
    printf("WarmUp: %f\n", ms > 0.f ? 1000.0f / ms : 0.f);
}

void cleanupCudaResources() {
  std::lock_guard<std::mutex> lk(g_mu);
  drop_secondary();
  if (g_scene) kdgr_scene_destroy(g_scene);
  g_scene = nullptr;
  g_have_frame = false;
  if (g_have_tree) kdgr_tree_free(&g_tree);
  g_have_tree = false;
}

int read_kd_tree_from_file(CompositeObject* object, const char* filename, int dump_format) {
  if (!object || !filename) return 0;
  std::lock_guard<std::mutex> lk(g_mu);
  kdgr_tree t;
  const bool binary = dump_format == KD_TREE_DUMP_IN_BINARY;
  if ((binary ? kdgr_read_kdt(filename, &t) : kdgr_read_kdt_ascii(filename, &t)) != KDGR_OK) {
    fprintf(stderr, "%s kd-tree File Load Error! (%s)\n", filename, kdgr_last_error());
    return 0;
  }
  if (g_have_tree) kdgr_tree_free(&g_tree);
  g_tree = t;
  g_have_tree = true;
  static KdTree kt;
  kt.tree = reinterpret_cast<KdTreeNode*>(g_tree.nodes);
  kt.tree_node_count = (int)g_tree.n_nodes;
  kt.prim_offset_list = g_tree.offsets;
  kt.prim_offset_count = (int)g_tree.n_offsets;
  if (binary) {
    // .kdt header order (xmin, ymin, zmin, xmax, ymax, zmax) -> AABB[XMIN..ZMAX]
    object->AABB[0] = g_tree.aabb[0];
    object->AABB[2] = g_tree.aabb[1];
    object->AABB[4] = g_tree.aabb[2];
    object->AABB[1] = g_tree.aabb[3];
    object->AABB[3] = g_tree.aabb[4];
    object->AABB[5] = g_tree.aabb[5];
  }
  memcpy(kt.AABB, object->AABB, sizeof(kt.AABB));
  object->kd_tree = &kt;
  return 1;
}

bool loadGaussiansFromPly(const char* filename, std::vector<Gaussian>& gaussians) {
  static_assert(sizeof(Gaussian) == 64 * sizeof(float), "Gaussian must be the reference's 64-float record");
  kdgr_gaussians g;
  if (!filename || kdgr_read_ply(filename, &g) != KDGR_OK) {
    fprintf(stderr, "Error: Cannot load PLY file %s (%s)\n", filename ? filename : "(null)", kdgr_last_error());
    return false;
  }
  gaussians.resize(g.n);
  memcpy(gaussians.data(), g.records, sizeof(Gaussian) * (size_t)g.n);
  kdgr_gaussians_free(&g);
  fprintf(stderr, "\nRobustly loaded %zu gaussians based on PLY header.\n", gaussians.size());
  return true;
}
