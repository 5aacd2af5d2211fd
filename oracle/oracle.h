/* oracle.h -- CPU restatement of the reference render kernel.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg load liboracle; the product (libkdgr) never
 * does and has no CPU render path.
 *
 * Two variants of one transcription of cudaRenderer.cu:
 *   f32: the oracle-matching build.  FP32, IEEE operations in the
 *        reference's order, no FMA contraction (-ffp-contract=off).  Its
 *        documented deviations from the reference GPU binary:
 *          __fdividef (cudaRenderer.cu:383-395,1560) -> IEEE division,
 *          rsqrtf in safe_normalize (:53-56)          -> 1.0f / sqrtf,
 *          CUDA expf in particleResponse (:678)       -> kdgr_expf
 *          (3dgrt_kdtree_gb300/csrc/kdgr_math.h, shared with the device).
 *   f64: the same algorithm in double precision with libm exp; the accuracy
 *        reference for the fast and reduced-precision forms.
 *
 * Parity pinning: the reference has no tests, golden images or vectors for
 * this path.  The transcription is pinned by the known-answer tests in
 * tests/test_oracle.py (analytic single-Gaussian cases) and runs on trees
 * the reference's own builder writes (oracle/build_ref.sh).
 */
#ifndef KDGR_ORACLE_H_
#define KDGR_ORACLE_H_

#include <stdint.h>

#include "kdgr.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  const uint32_t* nodes; /* 2 words per node, reference layout */
  uint32_t n_nodes;
  const uint32_t* offsets;
  uint32_t n_offsets;
  float aabb[6];         /* .kdt order: xmin, ymin, zmin, xmax, ymax, zmax */
  const float* gauss;    /* 64-float records, scale[] ALREADY INVERTED (1/s)
                            as the reference uploads them
                            (Kd-treeConverterMain.cpp:3636-3650) */
  uint32_t n_gauss;
} orc_scene;

/* CameraInfo of cudaRenderer.cu:336 (eye, u, v, startPoint, stepX, stepY). */
typedef struct {
  float eye[3], u[3], v[3], start[3];
  float step_x, step_y;
} orc_caminfo;

/* The host camera set-up of renderGaussianWithCudaFrame
 * (cudaRenderer.cu:3112-3127), same types and operation order. */
void orc_caminfo_from_camera(const kdgr_camera* cam, int width, int height, orc_caminfo* out);

/* Render the listed pixels (index y*width + x, y counted from the top row the
 * kernel's thread y addresses).  Outputs are per list entry: rgb[3*i..],
 * alpha[i], depth[i]; trace[i] when non-null.  threads <= 0: all. */
int orc_render_f32(const orc_scene* s, const orc_caminfo* c, int width, int height, const uint32_t* pix,
                   uint32_t n_pix, float* rgb, float* alpha, float* depth, kdgr_ray_trace* trace, int threads);
int orc_render_f64(const orc_scene* s, const orc_caminfo* c, int width, int height, const uint32_t* pix,
                   uint32_t n_pix, double* rgb, double* alpha, double* depth, kdgr_ray_trace* trace, int threads);

/* The secondary-ray kernel (renderKernelGaussian_Mesh_Hybrid), FP32
 * oracle-matching; spheres 10 floats each (center, radius, material word as
 * int bits, reflectivity, ior, color), triangles 9 floats each with one
 * 6-float material.  rgb per list entry, clamped to <= 1. */
int orc_render_hybrid_f32(const orc_scene* s, const orc_caminfo* c, int width, int height, const uint32_t* pix,
                          uint32_t n_pix, const float* spheres, int n_spheres, const float* tris, uint32_t n_tris,
                          const float* tri_material, float* rgb, int threads);

/* kdgr_expf, exported for the error test. */
float orc_expf(float x);
/* The same over an array. */
void orc_expf_n(const float* x, float* y, uint32_t n);

#ifdef __cplusplus
}
#endif
#endif /* KDGR_ORACLE_H_ */
