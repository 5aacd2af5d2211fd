// kdgr_api.cpp -- C ABI: device selection, scene upload, plain render calls.
//
// Scene upload replaces renderGaussianWithCudaSetup (cudaRenderer.cu:
// 2557-2703): where the reference copies the tree and the 256-byte AoS
// Gaussians once and binds texture objects (then destroys them, :2693-2702),
// this validates the tree, builds the device layouts each render form reads
// (see device_common.cuh) and keeps them for the scene's lifetime.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <deque>
#include <memory>
#include <string>
#include <vector>

#include "kdgr_internal.h"
#include "scene.h"

namespace kdgr {

int cuda_fail(cudaError_t e, const char* where) {
  set_error(std::string(where) + ": " + cudaGetErrorString(e));
  cudaGetLastError();  // clear a sticky launch-configuration error
  return e == cudaErrorMemoryAllocation ? KDGR_ERR_OUT_OF_MEMORY : KDGR_ERR_CUDA;
}

CamInfo make_caminfo(const kdgr_camera& cam, int width, int height) {
  CamInfo c;
  const float kPi = 3.14159265358979323846f;  // M_PI as cudaRenderer.h:31 defines it
  const float fov_rad = (float)(cam.fovy * (kPi / 180.0f));
  const float plane_height = (float)(2.0f * cam.near_c * tanf(fov_rad * 0.5f));
  const float plane_width = (float)(plane_height * cam.aspect);
  c.step_x = plane_width / width;
  c.step_y = plane_height / height;
  const float nc = (float)cam.near_c;
  for (int i = 0; i < 3; ++i) {
    c.eye[i] = cam.pos[i];
    c.u[i] = cam.uaxis[i];
    c.v[i] = cam.vaxis[i];
    const float a = cam.pos[i] - cam.naxis[i] * nc;
    const float b = a - cam.uaxis[i] * (plane_width * 0.5f);
    c.start[i] = b + cam.vaxis[i] * (plane_height * 0.5f);
  }
  return c;
}

void relayout_tree(const uint32_t* nodes, uint32_t n_nodes, int top_levels, std::vector<uint32_t>& out,
                   uint32_t* top_count) {
  std::vector<uint32_t> newidx(n_nodes, 0xFFFFFFFFu), order;
  order.reserve(n_nodes);
  struct Q {
    uint32_t old, depth;
  };
  std::deque<Q> q;
  newidx[0] = 0;
  order.push_back(0);
  q.push_back({0, 0});
  std::vector<uint32_t> frontier;  // inner nodes at depth == top_levels
  while (!q.empty()) {
    Q it = q.front();
    q.pop_front();
    const uint32_t x = nodes[2 * it.old];
    if ((x & 7u) == 3u) continue;
    if ((int)it.depth >= top_levels) {
      frontier.push_back(it.old);
      continue;
    }
    const uint32_t c = x >> 3;
    newidx[c] = (uint32_t)order.size();
    order.push_back(c);
    newidx[c + 1] = (uint32_t)order.size();
    order.push_back(c + 1);
    q.push_back({c, it.depth + 1});
    q.push_back({c + 1, it.depth + 1});
  }
  *top_count = (uint32_t)order.size();
  std::vector<uint32_t> st;
  for (uint32_t f : frontier) {
    st.push_back(f);
    while (!st.empty()) {
      const uint32_t o = st.back();
      st.pop_back();
      const uint32_t x = nodes[2 * o];
      if ((x & 7u) == 3u) continue;
      const uint32_t c = x >> 3;
      newidx[c] = (uint32_t)order.size();
      order.push_back(c);
      newidx[c + 1] = (uint32_t)order.size();
      order.push_back(c + 1);
      st.push_back(c + 1);
      st.push_back(c);
    }
  }
  out.assign(2 * (size_t)order.size(), 0);
  for (size_t n = 0; n < order.size(); ++n) {
    const uint32_t o = order[n];
    const uint32_t x = nodes[2 * o], y = nodes[2 * o + 1];
    if ((x & 7u) == 3u) {
      out[2 * n] = x;
      out[2 * n + 1] = y;
    } else {
      out[2 * n] = (newidx[x >> 3] << 3) | (x & 3u);
      out[2 * n + 1] = y;
    }
  }
}

void pad_leaf_pairs(std::vector<uint32_t>& relaid, const uint32_t* offsets, std::vector<uint32_t>& pair_gid) {
  pair_gid.clear();
  for (size_t n = 0; 2 * n < relaid.size(); ++n) {
    const uint32_t x = relaid[2 * n];
    if ((x & 7u) != 3u) continue;
    const uint32_t cnt = x >> 3, off = relaid[2 * n + 1];
    relaid[2 * n + 1] = (uint32_t)(pair_gid.size() / 2);
    pair_gid.insert(pair_gid.end(), offsets + off, offsets + off + cnt);
    if (cnt & 1u) pair_gid.push_back(kPadGid);
  }
}

}  // namespace kdgr

using namespace kdgr;

kdgr::ExactView kdgr_scene_s::exact_view() const {
  ExactView v;
  v.nodes = d_nodes;
  v.offsets = d_offsets;
  v.test = d_test;
  v.sh = d_sh;
  v.n_nodes = n_nodes;
  v.n_offsets = n_offsets;
  v.n_gauss = n_gauss;
  for (int i = 0; i < 3; ++i) {
    v.bmin[i] = aabb[i];
    v.bmax[i] = aabb[3 + i];
  }
  return v;
}

kdgr::FastView kdgr_scene_s::fast_view(bool packed) const {
  FastView v;
  v.nodes = packed ? d_nodes_packed : d_nodes_fast;
  v.offsets = packed ? d_gid_plain : d_pair_gid;
  v.opacity = d_opacity;
  v.sh = d_sh;
  v.sh_bf16 = d_sh_bf16;
  v.leaf_pairs = packed ? d_flag_pairs : d_leaf_pairs;
  v.leaf_packed = d_leaf_packed;
  v.leaf_aux = packed ? d_leaf_aux : nullptr;
  v.flag_offsets = packed ? d_gid_flag : nullptr;
  v.n_nodes = n_nodes;
  v.n_offsets = packed ? n_plain_entries : n_pair_entries;
  v.n_flag = packed ? n_flag_entries : 0u;
  v.n_gauss = n_gauss;
  v.top_nodes = top_nodes;
  for (int i = 0; i < 3; ++i) {
    v.bmin[i] = aabb[i];
    v.bmax[i] = aabb[3 + i];
  }
  return v;
}

namespace {

constexpr int kTopLevels = 10;  // 2047 nodes at most = 16 KB of shared memory

}  // namespace

namespace kdgr {

// renderGaussianWithCudaSetup (cudaRenderer.cu:2557-2703) from device-resident
// 64-float records: the per-Gaussian arrays of every requested form are
// written by the packing kernel (scene_pack.cu), the tree is uploaded as
// given (plain form) and relaid out with its leaf-order pair records (fast
// forms).  The tree must have been validated.
int scene_create_impl(const uint32_t* nodes, uint32_t n_nodes, const uint32_t* offsets, uint32_t n_offsets,
                      const float aabb[6], const float* d_g, uint32_t n, uint32_t flags, uint32_t depth,
                      kdgr_scene_t* out, const char* who) {
  const std::string w(who);
  uint32_t forms = flags & (KDGR_FORM_EXACT | KDGR_FORM_FAST | KDGR_FORM_PACKED);
  if (forms == 0) forms = KDGR_FORM_EXACT | KDGR_FORM_FAST;
  const bool inverted = (flags & KDGR_SCALES_INVERTED) != 0;

  std::unique_ptr<kdgr_scene_s> s(new kdgr_scene_s);
  cudaGetDevice(&s->device);
  s->forms = forms;
  s->n_nodes = n_nodes;
  s->n_offsets = n_offsets;
  s->n_gauss = n;
  s->depth = depth;
  memcpy(s->aabb, aabb, sizeof(s->aabb));
  for (uint32_t i = 0; i < n_nodes; ++i)
    if ((nodes[2 * i] & 7u) == 3u) {
      ++s->n_leaves;
      if ((nodes[2 * i] >> 3) > s->max_leaf) s->max_leaf = nodes[2 * i] >> 3;
    }

  DevAlloc A;
  std::vector<void*> staging;
  auto fail = [&](const std::string& where, cudaError_t e = cudaSuccess) {
    if (e == cudaSuccess) e = A.err != cudaSuccess ? A.err : cudaGetLastError();
    for (void* p : staging) cudaFree(p);
    A.release();
    return cuda_fail(e, (w + ": " + where).c_str());
  };
  auto stage = [&](size_t bytes, void** p) {
    const cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
    if (e == cudaSuccess) staging.push_back(*p);
    return e;
  };
  s->d_offsets = A.alloc<uint32_t>(n_offsets ? n_offsets : 1);
  s->d_sh = A.alloc<float4>(12 * (size_t)n);
  s->d_status = A.alloc<uint32_t>(1);
  if (forms & KDGR_FORM_EXACT) {
    s->d_nodes = A.alloc<uint2>(n_nodes);
    s->d_test = A.alloc<float4>(4 * (size_t)n);
  }
  if (forms & (KDGR_FORM_FAST | KDGR_FORM_PACKED)) s->d_opacity = A.alloc<float>(n);
  if (forms & KDGR_FORM_PACKED) s->d_sh_bf16 = A.alloc<uint4>(6 * (size_t)n);
  if (A.err != cudaSuccess) return fail("cudaMalloc");
  if (n_offsets && cudaMemcpy(s->d_offsets, offsets, 4ull * n_offsets, cudaMemcpyHostToDevice) != cudaSuccess)
    return fail("upload offsets");
  if (s->d_nodes && cudaMemcpy(s->d_nodes, nodes, 8ull * n_nodes, cudaMemcpyHostToDevice) != cudaSuccess)
    return fail("upload nodes");
  if (cudaMemset(s->d_status, 0, 4) != cudaSuccess) return fail("status");

  // per-Gaussian arrays, packed on the device
  PackOut po{};
  po.sh = s->d_sh;
  po.test = s->d_test;
  po.opacity = s->d_opacity;
  po.sh_bf16 = s->d_sh_bf16;
  float* d_giscl = nullptr;
  float4* d_fast = nullptr;
  uint32_t* d_packed = nullptr;
  uint8_t* d_aniso = nullptr;
  cudaError_t e = stage(12ull * n, (void**)&d_giscl);
  if (e == cudaSuccess && (forms & KDGR_FORM_FAST)) e = stage(48ull * n, (void**)&d_fast);
  if (e == cudaSuccess && (forms & KDGR_FORM_PACKED)) e = stage(32ull * n, (void**)&d_packed);
  if (e == cudaSuccess && (forms & KDGR_FORM_PACKED)) e = stage(n, (void**)&d_aniso);
  if (e != cudaSuccess) return fail("cudaMalloc (staging)", e);
  po.giscl = d_giscl;
  po.fast = d_fast;
  po.packed = d_packed;
  po.aniso = d_aniso;
  e = launch_pack(d_g, n, inverted, po, nullptr);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return fail("packing kernel", e);

  std::vector<uint32_t> relaid, pair_gid;  // relaid fast tree, padded leaf order (fast forms)
  if (forms & (KDGR_FORM_FAST | KDGR_FORM_PACKED)) {
    relayout_tree(nodes, n_nodes, kTopLevels, relaid, &s->top_nodes);
    pad_leaf_pairs(relaid, offsets, pair_gid);
    if (pair_gid.size() > 0xFFFFFFF0ull) {
      for (void* p : staging) cudaFree(p);
      A.release();
      set_error(w + ": more than 2^32 leaf entries after pair padding");
      return KDGR_ERR_LIMIT;
    }
    s->n_pair_entries = (uint32_t)pair_gid.size();
    s->d_nodes_fast = A.alloc<uint2>(n_nodes);
    s->d_pair_gid = A.alloc<uint32_t>(pair_gid.size() + 2);
    if (A.err != cudaSuccess) return fail("cudaMalloc (tree)");
    if (cudaMemcpy(s->d_nodes_fast, relaid.data(), 8ull * n_nodes, cudaMemcpyHostToDevice) != cudaSuccess ||
        (!pair_gid.empty() && cudaMemcpy(s->d_pair_gid, pair_gid.data(), 4 * pair_gid.size(),
                                         cudaMemcpyHostToDevice) != cudaSuccess))
      return fail("upload (tree)");
  }
  if (forms & KDGR_FORM_FAST) {
    // the per-Gaussian rows are staging: the kernels read the leaf-order pairs
    s->d_leaf_pairs = A.alloc<float4>(6 * ((size_t)s->n_pair_entries / 2 + 1));
    if (A.err != cudaSuccess) return fail("cudaMalloc (fast)");
    e = build_leaf_pairs(s->d_pair_gid, s->n_pair_entries, d_fast, s->d_leaf_pairs);
    if (e != cudaSuccess) return fail("leaf pairs (fast)", e);
  }
  if (forms & KDGR_FORM_PACKED) {
    const int rc = pack_precision(s.get(), d_g, d_giscl, d_packed, d_aniso, relaid, pair_gid, A);
    if (rc != KDGR_OK) {
      for (void* p : staging) cudaFree(p);
      A.release();
      return rc;
    }
  }
  for (void* p : staging) cudaFree(p);
  s->device_bytes = A.bytes;
  A.ptrs.clear();  // ownership moves to the scene
  *out = s.release();
  return KDGR_OK;
}

}  // namespace kdgr

extern "C" {

int kdgr_init(int device) {
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return cuda_fail(e, "kdgr_init: cudaSetDevice");
  e = cudaFree(nullptr);
  if (e != cudaSuccess) return cuda_fail(e, "kdgr_init: context");
  return KDGR_OK;
}

int kdgr_shutdown(void) {
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return cuda_fail(e, "kdgr_shutdown");
  return KDGR_OK;
}

int kdgr_scene_create(const uint32_t* nodes, uint32_t n_nodes, const uint32_t* offsets, uint32_t n_offsets,
                      const float aabb[6], const float* g, uint32_t n, uint32_t flags, kdgr_scene_t* out) {
  if (!out || !nodes || !aabb || !g || n == 0 || n_nodes == 0 || (n_offsets && !offsets)) {
    set_error("kdgr_scene_create: null argument, no nodes or no Gaussians");
    return KDGR_ERR_INVALID_ARG;
  }
  *out = nullptr;
  std::string err;
  uint32_t depth = 0;
  int rc = validate_tree(nodes, n_nodes, offsets, n_offsets, n, err, &depth);
  if (rc != KDGR_OK) {
    set_error("kdgr_scene_create: " + err);
    return rc;
  }
  // the records go to the device as they are; the device packs every form
  float* d_rec = nullptr;
  cudaError_t e = cudaMalloc(&d_rec, 256ull * n);
  if (e == cudaSuccess) e = cudaMemcpy(d_rec, g, 256ull * n, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    if (d_rec) cudaFree(d_rec);
    return cuda_fail(e, "kdgr_scene_create: record upload");
  }
  rc = scene_create_impl(nodes, n_nodes, offsets, n_offsets, aabb, d_rec, n, flags, depth, out,
                         "kdgr_scene_create");
  cudaFree(d_rec);
  return rc;
}

int kdgr_scene_create_device(const uint32_t* nodes, uint32_t n_nodes, const uint32_t* offsets, uint32_t n_offsets,
                             const float aabb[6], const float* d_g, uint32_t n, uint32_t flags, kdgr_scene_t* out) {
  if (!out || !nodes || !aabb || !d_g || n == 0 || n_nodes == 0 || (n_offsets && !offsets)) {
    set_error("kdgr_scene_create_device: null argument, no nodes or no Gaussians");
    return KDGR_ERR_INVALID_ARG;
  }
  *out = nullptr;
  std::string err;
  uint32_t depth = 0;
  int rc = validate_tree(nodes, n_nodes, offsets, n_offsets, n, err, &depth);
  if (rc != KDGR_OK) {
    set_error("kdgr_scene_create_device: " + err);
    return rc;
  }
  return scene_create_impl(nodes, n_nodes, offsets, n_offsets, aabb, d_g, n, flags, depth, out,
                           "kdgr_scene_create_device");
}

int kdgr_scene_destroy(kdgr_scene_t s) {
  if (!s) return KDGR_ERR_INVALID_ARG;
  DeviceScope on(s->device);
  void* ps[] = {s->d_nodes,     s->d_offsets, s->d_test,      s->d_sh,          s->d_nodes_fast,
                s->d_opacity,   s->d_sh_bf16,     s->d_leaf_pairs,  s->d_leaf_packed, s->d_pair_gid,
                s->d_nodes_packed, s->d_leaf_aux, s->d_gid_plain, s->d_gid_flag, s->d_flag_pairs,
                s->d_status};
  cudaError_t first = cudaSuccess;
  for (void* p : ps)
    if (p) {
      cudaError_t e = cudaFree(p);
      if (first == cudaSuccess) first = e;
    }
  delete s;
  if (first != cudaSuccess) return cuda_fail(first, "kdgr_scene_destroy");
  return KDGR_OK;
}

int kdgr_scene_info_get(kdgr_scene_t s, kdgr_scene_info* out) {
  if (!s || !out) {
    set_error("kdgr_scene_info_get: null argument");
    return KDGR_ERR_INVALID_ARG;
  }
  out->n_nodes = s->n_nodes;
  out->n_offsets = s->n_offsets;
  out->n_gaussians = s->n_gauss;
  out->depth = s->depth;
  out->n_leaves = s->n_leaves;
  out->max_leaf = s->max_leaf;
  out->forms = s->forms;
  out->top_nodes = s->top_nodes;
  out->n_aniso = s->n_aniso;
  out->device_bytes = s->device_bytes;
  return KDGR_OK;
}

int kdgr_scene_status(kdgr_scene_t s, uint32_t* bits, int clear) {
  if (!s || !bits) {
    set_error("kdgr_scene_status: null argument");
    return KDGR_ERR_INVALID_ARG;
  }
  DeviceScope on(s->device);
  cudaError_t e = on.err;
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(bits, s->d_status, 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && clear) e = cudaMemset(s->d_status, 0, 4);
  if (e != cudaSuccess) return cuda_fail(e, "kdgr_scene_status");
  return KDGR_OK;
}

static int render_common(kdgr_scene_t s, const kdgr_camera* cam, int W, int H, float* rgb, float* alpha, float* depth,
                         kdgr_ray_trace* trace, void* stream, float* ms_out, const char* who) {
  if (!s || !cam || !rgb || W <= 0 || H <= 0) {
    set_error(std::string(who) + ": null scene/camera/output or empty image");
    return KDGR_ERR_INVALID_ARG;
  }
  if (!(s->forms & KDGR_FORM_EXACT)) {
    set_error(std::string(who) + ": scene was created without KDGR_FORM_EXACT");
    return KDGR_ERR_INVALID_ARG;
  }
  DeviceScope on(s->device);
  if (on.err != cudaSuccess) return cuda_fail(on.err, who);
  const cudaStream_t st = (cudaStream_t)stream;
  const CamInfo ci = make_caminfo(*cam, W, H);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (ms_out) {
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
  }
  cudaError_t e = launch_exact(s->exact_view(), ci, W, H, rgb, alpha, depth, trace, s->d_status, 8, st);
  if (e != cudaSuccess) {
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    return cuda_fail(e, who);
  }
  if (ms_out) {
    cudaEventRecord(e1, st);
    e = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    *ms_out = ms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return cuda_fail(e, who);
  }
  return KDGR_OK;
}

int kdgr_render(kdgr_scene_t s, const kdgr_camera* cam, int W, int H, float* rgb, float* alpha, float* depth,
                void* stream, float* ms_out) {
  return render_common(s, cam, W, H, rgb, alpha, depth, nullptr, stream, ms_out, "kdgr_render");
}

int kdgr_render_trace(kdgr_scene_t s, const kdgr_camera* cam, int W, int H, float* rgb, float* alpha, float* depth,
                      kdgr_ray_trace* trace, void* stream) {
  if (!trace) {
    set_error("kdgr_render_trace: null trace buffer");
    return KDGR_ERR_INVALID_ARG;
  }
  return render_common(s, cam, W, H, rgb, alpha, depth, trace, stream, nullptr, "kdgr_render_trace");
}

}  // extern "C"
