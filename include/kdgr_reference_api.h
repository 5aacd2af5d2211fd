/* kdgr_reference_api.h -- the reference's render entry points, with the
 * reference's C++ signatures, implemented over the C ABI of kdgr.h.
 *
 * A caller of the reference renderer (KC = Kd-treeConverter_v0.9/
 * Kd-treeConverter/ of hydarlisk/3dgrt_kdtree) keeps its own headers
 * (cudaRenderer.h, Kd-treeConverter.h, OpenGLStuffs.h) built with
 * PRIMITIVE_TYPE 2 and SECONDARY_RAY 0, drops cudaRenderer.cu from its build and
 * links libkdgr.so instead: the types below use the reference's struct tags and
 * layouts, so the mangled names and the argument layouts are the reference's.
 * A caller without the reference headers may include this header instead (never
 * both: the types would be defined twice).
 *
 * Semantics follow the reference: one global scene, device 0, Gaussians with
 * scale[] already inverted by the caller (Kd-treeConverterMain.cpp:3636-3650),
 * a row-flipped RGB framebuffer, FPS returned after an event sync.  Errors are
 * printed and returned (false / 0 / -1) instead of exit() (cudaRenderer.cu:25-31).
 */
#ifndef KDGR_REFERENCE_API_H_
#define KDGR_REFERENCE_API_H_

#include <cuda_runtime.h>

#include <vector>

/* KdTreeNode, KdTree, CompositeObject for PRIMITIVE_TYPE 2
 * (KC/Kd-treeConverter.h:282-316) */
typedef struct _KdTreeNode {
  unsigned int x;
  unsigned int y;
} KdTreeNode;

typedef struct _KdTree {
  KdTreeNode* tree;
  int tree_node_count;
  unsigned int* prim_offset_list;
  int prim_offset_count;
  float AABB[6];
} KdTree;

struct _ExtendedVertex;
typedef struct _CompositeObject {
  int n_triangles;
  float AABB[6]; /* XMIN, XMAX, YMIN, YMAX, ZMIN, ZMAX (KC/Kd-treeConverter.h:160-165) */
  struct _ExtendedVertex* extended_vertices;
  KdTree* kd_tree;
  void* leafDebug;
} CompositeObject;

/* Gaussian with QUATERNION true (KC/Kd-treeConverter.h:319-335), 256 bytes */
struct Gaussian {
  float pos[3];
  float opacity;
  float scale[3];
  float k_scale;
  float rot[4];
  float f_dc[3];
  float f_rest[45];
  float pad[4];
};

/* Camera (KC/OpenGLStuffs.h:21-28); GLfloat = float, GLdouble = double */
typedef struct _cam {
  float pos[3];
  float uaxis[3], vaxis[3], naxis[3];
  float mat[16];
  float mat_inv[16];
  int move, upanddown;
  double fovy, aspect, near_c, far_c;
} Camera;

#define KD_TREE_DUMP_IN_ASCII 0
#define KD_TREE_DUMP_IN_BINARY 1

/* SecondaryMesh of the SECONDARY_RAY build (KC/cudaRenderer.h:12-19): the
 * triangle soup (3 vertices per triangle) and its one material. */
struct SecondaryMesh {
  std::vector<float3> vert;
  int triangleCount = 0;
  int materialType = 1; /* 1: reflect, 2: refract, 0: opaque */
  float reflectivity = 0.95f;
  float ior = 1.1f;
  float3 color = {0.95f, 0.95f, 0.95f};
};

/* SECONDARY_PRIM values (KC/Kd-treeConverter.h:28-30) */
#define KDGR_SECONDARY_TRI 0
#define KDGR_SECONDARY_SPHERE 1

/* initCuda (KC/cudaRenderer.cu:2438-2455): device 0. */
bool initCuda();
/* renderGaussianWithCudaSetup (KC/cudaRenderer.cu:2557-2703), SECONDARY_RAY 0. */
void renderGaussianWithCudaSetup(const CompositeObject& object, const std::vector<Gaussian>& gaussians);
/* The SECONDARY_RAY build's setup (KC/cudaRenderer.h:91-97, cudaRenderer.cu:
 * 2557-2703 with initSecondaryMesh :2064-2083): the scene plus the secondary
 * mesh; later frames run the secondary-ray renderer (renderKernelGaussian_
 * Mesh_Hybrid) against the reference's demo spheres (SECONDARY_PRIM SPHERE,
 * the committed setting) or the mesh (SECONDARY_PRIM TRI), chosen with
 * setSecondaryPrimitive.  The mesh vertices are copied. */
void renderGaussianWithCudaSetup(const CompositeObject& object, const std::vector<Gaussian>& gaussians,
                                 SecondaryMesh& secondaryMesh);
/* Run-time stand-in for the reference's compile-time SECONDARY_PRIM
 * (KDGR_SECONDARY_SPHERE by default); not a reference function. */
void setSecondaryPrimitive(int prim);
/* The HIT_AND_NODE_COUNT_DEBUG build's per-frame report (KC/cudaRenderer.cu:
 * 3173-3400): with a directory set (here, or through the environment variable
 * KDGR_DEBUG_REPORT_DIR at setup), every frame also writes renderStats.txt,
 * render_stats.csv, the heatmaps and the count files there (kdgr_debug_report).
 * nullptr switches it off.  Not a reference function: the reference selects
 * this at compile time and writes to "../../output/". */
void setDebugReportDir(const char* dir);
/* renderGaussianWithCudaFrame (KC/cudaRenderer.cu:3099-3484): plain drop-in
 * (oracle-matching) kernel into d_framebuffer (3*width*height floats, rows
 * flipped); returns 1000 / kernel-ms. */
float renderGaussianWithCudaFrame(const Camera& camera, int width, int height, float* d_framebuffer,
                                  cudaStream_t stream);
/* warmUp (KC/cudaRenderer.cu:2532-2554): re-renders the last frame's camera and
 * size into d_framebuffer (no-op before the first frame). */
void warmUp(float* d_framebuffer, cudaStream_t stream);
/* cleanupCudaResources (KC/cudaRenderer.cu:3486-3521). */
void cleanupCudaResources();
/* read_kd_tree_from_file (KC/Kd-treeConverter.cpp:444-572), binary or ASCII
 * format (the ASCII format has no box: object->AABB is left as it was, as in
 * the reference); validates the tree.  Returns 1 on success, 0 otherwise.
 * The arrays are owned by the library until the next call or
 * cleanupCudaResources. */
int read_kd_tree_from_file(CompositeObject* object, const char* filename, int dump_format);
/* loadGaussiansFromPly (KC/Kd-treeConverterMain.cpp:1652-1769): a binary
 * little-endian 3DGS .ply into activated Gaussians (kdgr_read_ply). */
bool loadGaussiansFromPly(const char* filename, std::vector<Gaussian>& gaussians);

#endif /* KDGR_REFERENCE_API_H_ */
