// ref_kdbuild.cpp -- driver around the reference kd-tree builder.
// TEST INFRASTRUCTURE ONLY (the oracle side): it is linked with the
// reference's own Kd-treeConstructor.cpp / Kd-treeConverter.cpp /
// MyMathUtility.cpp, compiled where they lie by oracle/build_ref.sh, and
// produces the `.kdt` tree the reference would write for a scene.  The
// product's own builder is checked against the files this writes.
//
// The reference's headless build (`-t`, Kd-treeConverterMain.cpp:3738-3762)
// lives in a translation unit that needs GL/GLUT and <direct.h>, so the two
// steps of it that precede the builder are restated here:
//   * proxy mesh: create_composite_object_from_gaussians
//     (Kd-treeConverterMain.cpp:1925-2101, non-adaptive icosahedron branch
//     :2092-2095) with generate_gaussian_mesh (:1860-1922) and
//     rotate_vector_by_quaternion (:1623-1638);
//   * validity cut: sigma < KERNEL_MIN_RESPONSE || sigma < 1/255 drops the
//     Gaussian (:1990-1997).
// The build itself is the reference's build_kd_tree_for_composite_object
// (Kd-treeConverter.cpp:22) and the file is written by the reference's
// dump_kd_tree_for_composite_object (Kd-treeConverter.cpp:297-342).
//
// Input: a KDGS scene file (16-byte header "KDGS", u32 version 1, u32 n,
// u32 floats-per-record 64, then n activated Gaussian records in the
// reference's 256-byte `Gaussian` layout, Kd-treeConverter.h:319-335).

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "Kd-treeConverter.h"
#include "Kd-treeConstructor.h"
#include "MyMathUtility.h"

// Build parameters the reference keeps as globals in its main translation
// unit (Kd-treeConverterMain.cpp:46-61).  Defaults follow the reference; the
// command line overrides them like its -m/-f/-i/-s/-sc/-om flags
// (:3679-3733).
int MAX_LEVEL = 256;
float ISCET_COST = 5.0f;
int FORCE_SPLIT_THRESHOLD = 256;
int SAH_MODE = 1;
int OFFSET_MAX = 2;
float SORT_COST = 0.5f;
std::vector<Gaussian> g_gaussians;
std::vector<bool> g_isValidG;

static const float kIcoVerts[12][3] = {
    {-1.f, 1.618033988749895f, 0.f}, {1.f, 1.618033988749895f, 0.f},
    {0.f, 1.f, -1.618033988749895f}, {-1.618033988749895f, 0.f, -1.f},
    {-1.618033988749895f, 0.f, 1.f}, {0.f, 1.f, 1.618033988749895f},
    {1.618033988749895f, 0.f, 1.f},  {0.f, -1.f, 1.618033988749895f},
    {-1.f, -1.618033988749895f, 0.f}, {0.f, -1.f, -1.618033988749895f},
    {1.618033988749895f, 0.f, -1.f}, {1.f, -1.618033988749895f, 0.f}};
static const int kIcoFaces[20][3] = {
    {0, 1, 2},  {0, 2, 3},  {0, 3, 4},  {0, 4, 5},  {0, 5, 1},
    {6, 1, 5},  {6, 5, 7},  {6, 7, 11}, {6, 11, 10}, {6, 10, 1},
    {8, 4, 3},  {8, 3, 9},  {8, 9, 11}, {8, 11, 7}, {8, 7, 4},
    {9, 3, 2},  {9, 2, 10}, {9, 10, 11}, {5, 4, 7}, {1, 10, 2}};

// Min/max as the reference's main translation unit sees them: the overloads
// cudaRenderer.h:50-51 defines, which it includes (Kd-treeConverterMain.cpp:40).
static inline float ref_fminf(float a, float b) { return (b > a) ? a : b; }
static inline float ref_fmaxf(float a, float b) { return (b < a) ? a : b; }

static void rotate_by_quat(float out[3], const float v[3], const float q[4]) {
  float qv3[3] = {q[1], q[2], q[3]};
  float vv[3] = {v[0], v[1], v[2]};
  float t[3], tt[3];
  fMyVecCrossProduct(qv3, vv, t);
  for (int i = 0; i < 3; ++i) t[i] *= 2.0f;
  fMyVecCrossProduct(qv3, t, tt);
  for (int i = 0; i < 3; ++i) out[i] = vv[i] + q[0] * t[i] + tt[i];
}

static bool read_scene(const char* path, std::vector<Gaussian>& out) {
  FILE* fp = fopen(path, "rb");
  if (!fp) return false;
  char magic[4];
  uint32_t hdr[3];
  bool ok = fread(magic, 1, 4, fp) == 4 && memcmp(magic, "KDGS", 4) == 0 &&
            fread(hdr, 4, 3, fp) == 3 && hdr[0] == 1 && hdr[2] == 64;
  if (ok) {
    out.resize(hdr[1]);
    ok = fread(out.data(), sizeof(Gaussian), hdr[1], fp) == hdr[1];
  }
  fclose(fp);
  return ok;
}

int main(int argc, char** argv) {
  static_assert(sizeof(Gaussian) == 256, "Gaussian record must be 256 B");
  if (argc < 3) {
    fprintf(stderr, "usage: %s scene.kdgs out.kdt [-m L] [-f N] [-i C] [-s M] [-sc C] [-om K]\n", argv[0]);
    return 2;
  }
  for (int a = 3; a + 1 < argc; a += 2) {
    std::string k = argv[a];
    if (k == "-m") MAX_LEVEL = atoi(argv[a + 1]);
    else if (k == "-f") FORCE_SPLIT_THRESHOLD = atoi(argv[a + 1]);
    else if (k == "-i") ISCET_COST = (float)atof(argv[a + 1]);
    else if (k == "-s") SAH_MODE = atoi(argv[a + 1]);
    else if (k == "-sc") SORT_COST = (float)atof(argv[a + 1]);
    else if (k == "-om") OFFSET_MAX = atoi(argv[a + 1]);
  }
  if (!read_scene(argv[1], g_gaussians)) {
    fprintf(stderr, "cannot read scene %s\n", argv[1]);
    return 1;
  }
  auto t0 = std::chrono::steady_clock::now();
  const long n = (long)g_gaussians.size();
  g_isValidG.assign(n, true);
  CompositeObject obj;
  memset(&obj, 0, sizeof(obj));
  obj.extended_vertices = (ExtendedVertex*)malloc(sizeof(ExtendedVertex) * 60 * (size_t)(n > 0 ? n : 1));
  obj.AABB[XMIN] = obj.AABB[YMIN] = obj.AABB[ZMIN] = FLT_MAX;
  obj.AABB[XMAX] = obj.AABB[YMAX] = obj.AABB[ZMAX] = -FLT_MAX;
  ExtendedVertex* vp = obj.extended_vertices;
  long ntri = 0;
  const float kMin = KERNEL_MIN_RESPONSE;
  for (long i = 0; i < n; ++i) {
    const Gaussian& g = g_gaussians[i];
    const float sigma = g.opacity;
    if (sigma < kMin || sigma < 1 / 255.0f) {
      g_isValidG[i] = false;
      continue;
    }
    float k_iso = 0.0f;
    if (sigma / kMin > 1.0f) k_iso = sqrtf(2.0f * logf(sigma / kMin)) * 0.5257311121191335703f;
    const float fs[3] = {g.scale[0] * k_iso, g.scale[1] * k_iso, g.scale[2] * k_iso};
    for (int f = 0; f < 20; ++f) {
      for (int l = 0; l < 3; ++l) {
        const float* vc = kIcoVerts[kIcoFaces[f][l]];
        float vs[3] = {vc[0] * fs[0], vc[1] * fs[1], vc[2] * fs[2]};
        float vr[3];
        rotate_by_quat(vr, vs, g.rot);
        float vf[3] = {vr[0] + g.pos[0], vr[1] + g.pos[1], vr[2] + g.pos[2]};
        memcpy(vp->vertex, vf, sizeof(vf));
        vp->material_ID = (int)i;
        float nrm[3] = {vf[0] - g.pos[0], vf[1] - g.pos[1], vf[2] - g.pos[2]};
        fMyVecNormalize(nrm);
        memcpy(vp->normal, nrm, sizeof(nrm));
        obj.AABB[XMIN] = ref_fminf(obj.AABB[XMIN], vf[0]);
        obj.AABB[XMAX] = ref_fmaxf(obj.AABB[XMAX], vf[0]);
        obj.AABB[YMIN] = ref_fminf(obj.AABB[YMIN], vf[1]);
        obj.AABB[YMAX] = ref_fmaxf(obj.AABB[YMAX], vf[1]);
        obj.AABB[ZMIN] = ref_fminf(obj.AABB[ZMIN], vf[2]);
        obj.AABB[ZMAX] = ref_fmaxf(obj.AABB[ZMAX], vf[2]);
        ++vp;
      }
    }
    ntri += 20;
  }
  obj.n_triangles = (int)ntri;
  auto t1 = std::chrono::steady_clock::now();
  if (!build_kd_tree_for_composite_object(&obj)) {
    fprintf(stderr, "reference build failed\n");
    return 1;
  }
  auto t2 = std::chrono::steady_clock::now();
  dump_kd_tree_for_composite_object(&obj, KD_TREE_DUMP_IN_BINARY, argv[2], "", nullptr);
  double proxy_s = std::chrono::duration<double>(t1 - t0).count();
  double build_s = std::chrono::duration<double>(t2 - t1).count();
  printf("KDGR_REF_RESULT {\"n_gauss\": %ld, \"n_triangles\": %ld, \"n_nodes\": %d, \"n_offsets\": %d, "
         "\"proxy_s\": %.6f, \"build_s\": %.6f}\n",
         n, ntri, obj.kd_tree->tree_node_count, obj.kd_tree->prim_offset_count, proxy_s, build_s);
  return 0;
}
