// device_common.cuh -- types shared by the render kernels and the host API.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "kdgr.h"

namespace kdgr {

// CameraInfo of the reference (cudaRenderer.cu:336): eye, right/up axes,
// top-left point of the near-plane window and the per-pixel steps.
struct CamInfo {
  float eye[3], u[3], v[3], start[3];
  float step_x, step_y;
};

// The host camera set-up of renderGaussianWithCudaFrame
// (cudaRenderer.cu:3112-3127) in the reference's types and order.
CamInfo make_caminfo(const kdgr_camera& cam, int width, int height);

// Device arrays of the oracle-matching (plain drop-in) form.
//   nodes:   the reference's 8-byte nodes, in the file's order;
//   offsets: leaf Gaussian-ID lists;
//   test:    4 x float4 per Gaussian, the fields the ray-Gaussian test reads:
//            (pos.xyz, opacity) (1/s.xyz, s.x) (s.y, s.z, q.w, q.x) (q.y, q.z, 0, 0)
//            with 1/s the reference's uploaded (inverted) scale and s its
//            IEEE reciprocal, the value rayPrimIntersect computes per call;
//   sh:      12 x float4 per Gaussian, coefficient-major RGB (k*3 + c).
struct ExactView {
  const uint2* nodes;
  const uint32_t* offsets;
  const float4* test;
  const float4* sh;
  uint32_t n_nodes, n_offsets, n_gauss;
  float bmin[3], bmax[3];
};

// Device arrays of one fast form (kdgr_scene_s::fast_view(packed)).
//   nodes:      re-laid-out tree: the top levels breadth-first, the rest
//               depth-first by subtree; children stay pairwise adjacent.
//               Leaf words: x = count << 3 | 3, y = the leaf's first pair p
//               of the main stream; its entries are 2p .. 2p + count - 1,
//               and an odd count ends with one padding entry.  The packed
//               form has its own leaf words: count and pairs cover only the
//               leaf's plain entries;
//   offsets:    Gaussian ID of every main-stream entry in that padded leaf
//               order (0xFFFFFFFF for padding), read for accepted hits only;
//               n_offsets counts them;
//   opacity:    1 float per Gaussian;
//   sh:         FP32 coefficient-major (shared with ExactView);
//   sh_bf16:    6 x uint4 per Gaussian, BF16 coefficient-major;
//   leaf_pairs: FP32 pairs: per pair of entries (2p, 2p+1) the rows of
//               M = diag(1/s) R^T and b = M mu interleaved lo/hi, 6 x float4.
//               The FP32 form's main stream; in the packed form the stream of
//               flagged entries (scale ratio > 1e3, or factors beyond FP16),
//               whose rows come from the FP64 upload precompute;
//   leaf_packed: packed form, per pair of plain entries 4 x uint4: the FP32
//               means and the FP16 entries of M interleaved lo/hi;
//   leaf_aux:   packed form, per node: at a leaf (first flagged pair, number
//               of flagged entries); flag_offsets their Gaussian IDs (n_flag).
//   A leaf's hit index runs over its main-stream entries, then (packed) its
//   flagged entries.  Padding entries hold zero records: M = 0 gives
//   |grdu|^2 = 0 and t* = 0 * inf = NaN, which no leaf interval accepts.
struct FastView {
  const uint2* nodes;
  const uint32_t* offsets;
  const float* opacity;
  const float4* sh;
  const uint4* sh_bf16;
  const float4* leaf_pairs;     // FP32 pairs (6 x float4): the FP32 form's leaf entries, or the
                                //   packed form's flagged entries
  const uint4* leaf_packed;     // packed form: FP16 pairs of the plain entries
  const uint2* leaf_aux;        // packed form, per node: (first flagged pair, n_flagged) at leaves
  const uint32_t* flag_offsets; // packed form: Gaussian of every padded flagged entry
  uint32_t n_nodes, n_offsets, n_flag, n_gauss, top_nodes;
  float bmin[3], bmax[3];
};

// One view of a batch: camera, image size, its work-item grids and where its
// pixels go in the output buffers.  Work items are 8x4-pixel warp tiles
// (per-warp scheduling) or 16x8-pixel CTA blocks (per-CTA scheduling).
struct ViewDesc {
  CamInfo cam;
  int32_t W, H;
  uint32_t wt_x, wt_base;  // 8x4 tiles per row; first global tile of the view
  uint32_t cb_x, cb_base;  // 16x8 blocks per row; first global block
  uint64_t out_off;
  uint32_t scene;          // scene slot (multi-scene launches of the serving loop)
  uint32_t pad;
};

__host__ __device__ inline uint64_t fnv_add(uint64_t h, uint32_t v) {
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    h ^= (v >> (8 * i)) & 0xFFu;
    h *= 1099511628211ull;
  }
  return h;
}
constexpr uint64_t kFnvInit = 14695981039346656037ull;

// Error bits a kernel writes to its status word (never traps).
enum : uint32_t {
  kStatusBadNode = 1u,     // child index outside the node array
  kStatusBadLeaf = 2u,     // leaf range outside the ID array
  kStatusBadId = 4u,       // Gaussian ID >= n_gauss
  kStatusQueueTimeout = 8u, // a bounded queue wait expired
  kStatusStepLimit = 16u    // a ray exceeded kMaxRaySteps node fetches
};

// Upper bound on node fetches per ray.  A valid tree needs far fewer (each
// leaf is entered once per restart and restarts strictly advance t_near);
// the bound only guarantees that a kernel on a malformed input ends.
constexpr uint32_t kMaxRaySteps = 1u << 22;

// Launch entry points (render_exact.cu).
// Secondary primitives of the hybrid kernel, device arrays:
//   spheres: 10 floats each (center xyz, radius, material word, reflectivity,
//            ior, color rgb); the material word is an int stored bitwise;
//   tris:    9 floats each (three vertices), one material for all of them
//            (tri_material: the 6 material floats, device pointer).
struct HybridView {
  const float* spheres;
  const float* tris;
  const float* tri_material;
  int n_spheres;
  uint32_t n_tris;
};

cudaError_t launch_hybrid(const ExactView& s, const CamInfo& cam, int width, int height, const HybridView& m,
                          float* rgb, uint32_t* status, cudaStream_t stream);

cudaError_t launch_exact(const ExactView& s, const CamInfo& cam, int width, int height, float* rgb, float* alpha,
                         float* depth, kdgr_ray_trace* trace, uint32_t* status, int kbuf, cudaStream_t stream);

}  // namespace kdgr
