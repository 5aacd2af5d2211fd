// scene.h -- the scene handle behind kdgr_scene_t (host side).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <mutex>
#include <string>
#include <vector>

#include "device_common.cuh"
#include "kdgr.h"

struct kdgr_scene_s {
  int device = 0;
  uint32_t forms = 0;  // KDGR_FORM_* materialised on the device
  uint32_t n_nodes = 0, n_offsets = 0, n_gauss = 0;
  uint32_t depth = 0, max_leaf = 0, n_leaves = 0;
  float aabb[6] = {0, 0, 0, 0, 0, 0};  // .kdt order
  // oracle-matching form
  uint2* d_nodes = nullptr;
  uint32_t* d_offsets = nullptr;
  float4* d_test = nullptr;
  float4* d_sh = nullptr;
  // fast forms
  uint2* d_nodes_fast = nullptr;
  uint32_t top_nodes = 0;
  float* d_opacity = nullptr;
  uint4* d_sh_bf16 = nullptr;
  // leaf-major copies of the test records, padded per leaf to whole pairs:
  // the fast tree's leaf word y is the leaf's first pair p, its entries are
  // 2p .. 2p+cnt-1 and an odd leaf ends with one padding entry;
  // d_pair_gid[j] is the Gaussian of entry j (kPadGid for padding, whose
  // records are zero)
  uint32_t* d_pair_gid = nullptr;
  uint32_t n_pair_entries = 0;     // even
  float4* d_leaf_pairs = nullptr;  // FP32 form, 6 x float4 per pair of entries
  uint4* d_leaf_packed = nullptr;  // packed form, 4 x uint4 per pair of plain entries
  // The packed form's own leaf layout: a leaf's plain entries in FP16 pairs
  // (d_leaf_packed), its flagged entries (scale ratio > 1e3 or factors beyond
  // FP16: FP64-precomputed factors) in FP32 pairs of a second stream.
  uint2* d_nodes_packed = nullptr;  // leaf words (n_plain << 3 | 3, first plain pair)
  uint2* d_leaf_aux = nullptr;      // per node; at leaves (first flagged pair, n_flagged)
  uint32_t* d_gid_plain = nullptr;  // Gaussian of every padded plain entry
  uint32_t* d_gid_flag = nullptr;   // Gaussian of every padded flagged entry
  float4* d_flag_pairs = nullptr;   // 6 x float4 per flagged pair (FP32 pair layout)
  uint32_t n_plain_entries = 0, n_flag_entries = 0;
  uint32_t n_aniso = 0;
  // per-scene status word written by kernels (error bits)
  uint32_t* d_status = nullptr;
  size_t device_bytes = 0;
  std::mutex mu;

  kdgr::ExactView exact_view() const;
  kdgr::FastView fast_view(bool packed) const;
};

namespace kdgr {
// Makes `device` current for the enclosing scope and restores the caller's
// device afterwards: every call on a scene runs on the device the scene was
// created on, whatever device the calling thread has selected.
struct DeviceScope {
  int prev = -1;
  cudaError_t err = cudaSuccess;
  explicit DeviceScope(int device) {
    err = cudaGetDevice(&prev);
    if (err == cudaSuccess && prev != device) err = cudaSetDevice(device);
    else prev = -1;  // nothing to restore
  }
  ~DeviceScope() {
    if (prev >= 0) cudaSetDevice(prev);
  }
  DeviceScope(const DeviceScope&) = delete;
  DeviceScope& operator=(const DeviceScope&) = delete;
};

// Allocation helper that records bytes and frees everything on failure.
struct DevAlloc {
  std::vector<void*> ptrs;
  size_t bytes = 0;
  cudaError_t err = cudaSuccess;
  template <typename T>
  T* alloc(size_t count) {
    if (err != cudaSuccess) return nullptr;
    void* p = nullptr;
    const size_t b = count * sizeof(T) + 16;
    err = cudaMalloc(&p, b);
    if (err != cudaSuccess) return nullptr;
    ptrs.push_back(p);
    bytes += b;
    return static_cast<T*>(p);
  }
  void release() {
    for (void* p : ptrs) cudaFree(p);
    ptrs.clear();
  }
};

int cuda_fail(cudaError_t e, const char* where);
// Fast-form tree relayout: top levels breadth-first, rest depth-first.
void relayout_tree(const uint32_t* nodes, uint32_t n_nodes, int top_levels, std::vector<uint32_t>& out,
                   uint32_t* top_count);
// Packed precision form from the packing kernel's outputs: the FP64
// upload-time factors of flagged Gaussians and the form's own leaf layout.
int pack_precision(kdgr_scene_s* s, const float* d_rec, const float* d_giscl, const uint32_t* d_packed,
                   const uint8_t* d_aniso, const std::vector<uint32_t>& relaid,
                   const std::vector<uint32_t>& pair_gid, DevAlloc& A);
// Fast-form leaf layout: rewrites the leaf words of the relaid tree
// (y = first pair) and returns the padded per-entry Gaussian IDs.
void pad_leaf_pairs(std::vector<uint32_t>& relaid, const uint32_t* offsets, std::vector<uint32_t>& pair_gid);
constexpr uint32_t kPadGid = 0xFFFFFFFFu;
// Pair records in padded leaf order (entry j = Gaussian gid[j], zero for
// padding): FP32 from 3 float4 per Gaussian (rows of M and b), packed from
// 8 words per Gaussian, flagged FP32 pairs from the FP64-precomputed table
// (entry aidx[gid]).  The packed builders do not synchronize.
cudaError_t build_leaf_pairs(const uint32_t* d_gid, uint32_t n_entries, const float4* test, float4* pairs);
cudaError_t build_packed_pairs(const uint32_t* d_gid, uint32_t n_entries, const uint32_t* src, uint4* pairs);
cudaError_t build_flag_pairs(const uint32_t* d_gid, uint32_t n_entries, const uint32_t* aidx, const float4* table,
                             float4* pairs);
// Batched rendering (render_fast.cu).
// totals: 8x4 tiles, 16x8 blocks and 32x16 super-blocks over all views.
int make_view_table(const kdgr_view* views, int n_views, std::vector<ViewDesc>& out, uint32_t totals[3]);
int fill_view_table(const kdgr_view* views, int n_views, ViewDesc* out, uint32_t totals[3]);
int check_batch_config(kdgr_scene_t s, const kdgr_batch_config& c);
// Work-queue words of a batched launch: word 0 the global counter, words
// 1..kMaxStrips the per-SM strip counters (zero before every launch).
constexpr int kMaxStrips = 255;
constexpr size_t kQueueBytes = (1 + kMaxStrips) * sizeof(uint32_t);
cudaError_t launch_batch(kdgr_scene_t s, const kdgr_batch_config& c, const ViewDesc* d_views, int n_views,
                         const uint32_t totals[3], float* rgb, float* alpha, float* depth, uint32_t* queue,
                         cudaStream_t st);
int batch_sms();
// Writes a launch's view table to d_views and zeroes its queue words
// (kQueueBytes at d_queue), stream-ordered: up to 256 views in the
// parameters of one staging kernel, more by one copy from host memory that
// must stay valid until the copy has run.
cudaError_t stage_views(const ViewDesc* views, int n_views, ViewDesc* d_views, uint32_t* d_queue, cudaStream_t st);
// The serving loop's scene slots, passed whole in the parameters of each
// multi-scene launch (7.7 KB): a warp reads its scene's fields from the
// constant bank rather than from a table in global memory.
constexpr int kSceneSlots = 64;
struct SceneTable {
  FastView s[kSceneSlots];
};
// Multi-scene persistent launch (warp-strip schedule) for the serving loop;
// views[v].scene indexes the table and d_outs[v] is view v's output base.
cudaError_t launch_multi(const SceneTable& scenes, bool packed, const ViewDesc* d_views, int n_views,
                         uint32_t total_blocks, float* const* d_outs, uint32_t* queue, uint32_t* status,
                         cudaStream_t st);
// Scale ratio above which a Gaussian's factors come from the FP64 precompute.
constexpr double kAnisoRatio = 1e3;

// Per-Gaussian outputs of the device packing kernel (scene_pack.cu); a null
// pointer skips that output.
struct PackOut {
  float* giscl;         // 3 per Gaussian: inverse scale as uploaded by the reference's caller
  float4* sh;           // 12 per Gaussian: FP32 SH, coefficient-major
  float4* test;         // 4 per Gaussian: the plain kernel's test record
  float4* fast;         // 3 per Gaussian: rows of M and b (FP64 -> FP32)
  float* opacity;       // 1 per Gaussian
  uint32_t* packed;     // 8 per Gaussian: FP32 mean + FP16 entries of M (precision form staging)
  uint4* sh_bf16;       // 6 per Gaussian: BF16 SH, coefficient-major
  uint8_t* aniso;       // 1 per Gaussian (with packed): takes the FP64-precomputed factors
};
cudaError_t launch_pack(const float* d_rec, uint32_t n, bool inverted, const PackOut& out, cudaStream_t st);
// Fields of the FP64 precompute (k_aniso_fp64) for each flagged Gaussian i,
// written to entry aidx[i] of d_out (10 floats each; aidx 0xFFFFFFFF skips).
cudaError_t launch_gather_aniso(const float* d_rec, const float* d_giscl, const uint32_t* d_aidx, uint32_t n,
                                float* d_out, cudaStream_t st);

// Byte offsets within a PLY vertex of x, y, z, opacity, scale_0..2,
// rot_0..3, f_dc_0..2 and f_rest_0 (-1 when the file has no f_rest).
struct PlyLayout {
  int off[16];
};
// Parse a 3DGS .ply header (binary little-endian, float fields found by
// name); leaves fp at the first vertex.
int parse_ply_header(FILE* fp, PlyLayout& lay, uint64_t& n_vertices, uint32_t& stride, std::string& err);
cudaError_t launch_ply_activate(const uint8_t* d_raw, uint32_t n, uint32_t stride, const PlyLayout& lay,
                                float* d_rec, cudaStream_t st);
// Device records -> scene (all forms); the tree arrays are host arrays,
// validated by the caller.
int scene_create_impl(const uint32_t* nodes, uint32_t n_nodes, const uint32_t* offsets, uint32_t n_offsets,
                      const float aabb[6], const float* d_gaussians, uint32_t n, uint32_t flags, uint32_t depth,
                      kdgr_scene_t* out, const char* who);
}  // namespace kdgr
