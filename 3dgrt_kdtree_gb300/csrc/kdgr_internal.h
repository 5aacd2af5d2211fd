// kdgr_internal.h -- declarations shared by the host-side translation units
// of libkdgr (not part of the public C ABI; that is include/kdgr.h).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace kdgr {

struct BuildParams {
  int max_level = 24;     // -m  (MAX_LEVEL)
  int force_split = 16;   // -f  (FORCE_SPLIT_THRESHOLD, triangles)
  float isect_cost = 5.0f;  // -i (ISCET_COST)
  int sah_mode = 1;       // -s  (SAH_MODE)
  float sort_cost = 0.5f; // -sc (SORT_COST)
  int threads = 0;        // 0: hardware concurrency
};

struct BuildStats {
  double proxy_s = 0, build_s = 0, serialize_s = 0;
  uint64_t n_triangles = 0;
  uint32_t n_valid = 0;
};

// A kd-tree in the reference's flat layout: 8-byte nodes (two u32 words
// each) and the leaf Gaussian-ID array.  aabb is in `.kdt` header order
// (xmin, ymin, zmin, xmax, ymax, zmax).
struct HostTree {
  std::vector<uint32_t> nodes;    // 2 * n_nodes words
  std::vector<uint32_t> offsets;  // leaf ID lists
  float aabb[6] = {0, 0, 0, 0, 0, 0};
  uint32_t depth = 0, n_leaves = 0, max_leaf = 0;
  std::vector<uint8_t> valid;     // per Gaussian: 1 if it has proxy triangles
};

int build_tree(const float* gauss, uint32_t n, const BuildParams& bp, HostTree& out, BuildStats* stats);
bool proxy_icosahedron(const float* g, float out[20][3][3]);
// Proxy scale k_iso of one Gaussian; false when the opacity cut drops it.
bool proxy_kiso(const float* g, float* k_iso);
// Unit icosahedron of the proxy mesh (Kd-treeConverterMain.cpp:1860-1922).
extern const float kIcosaVerts[12][3];
extern const int kIcosaFaces[20][3];
// The same build on the current CUDA device (kdbuild_gpu.cu).
int build_tree_gpu(const float* gauss, uint32_t n, const BuildParams& bp, HostTree& out, BuildStats* stats,
                   std::string& err);

// .kdt v1 binary (Kd-treeConverter.cpp:297-342, 444-495)
int write_kdt(const HostTree& t, const char* path, std::string& err);
int read_kdt(const char* path, HostTree& t, std::string& err);
int write_kdt_ascii(const HostTree& t, const char* path, std::string& err);
int read_kdt_ascii(const char* path, HostTree& t, std::string& err);
// Structural validation: child indices in range, leaf ranges inside the
// ID array, IDs below n_gaussians, every node reachable at most once.
int validate_tree(const uint32_t* nodes, uint32_t n_nodes, const uint32_t* offsets, uint32_t n_offsets,
                  uint32_t n_gaussians, std::string& err, uint32_t* depth_out);

// Thread-local last-error text behind kdgr_last_error().
void set_error(const std::string& msg);

}  // namespace kdgr
