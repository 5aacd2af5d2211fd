// kdgr_noalloc.cu -- kdgr_render_batch_noalloc: the batched render call for
// callers that cannot allocate device memory.
//
// kdgr_render_batch takes its scratch -- the per-view table the persistent
// kernel reads and the atomic work-queue counter -- from the stream-ordered
// allocator on every call.  Some callers must not allocate at all: a host
// application that owns the whole device-memory budget and forbids libraries
// from taking more (or runs under a hard cap that an allocation could
// exceed), or a frame loop that must not enter the allocator, where an
// allocation can synchronise or fail from fragmentation at the worst moment.
// For them this entry point renders with the same kernel, but its scratch
// lives in one fixed, file-scope __device__ array: 32 KiB, enough for 256
// views.  Every GPU that loads the library holds that array until the
// process exits.
//
// Host code cannot pass the array's name to a kernel: on the host that name
// is only a stand-in, not a device address.  The first call on each device
// therefore asks the runtime for the array's device address
// (cudaGetSymbolAddress) with that device current and caches it; make that
// first call before any stream capture.  The call runs on the scene's device
// (it switches to it and back).
//
// The view table reaches the array inside the parameters of a one-block
// staging kernel (k_noalloc_stage, 24.6 KB of parameters; kernels take up to
// 32,764 bytes), which also zeroes the queue counter: nothing the call
// enqueues refers to host memory after it returns.  All calls share the
// array and it keeps the previous call's contents; each call rewrites the
// table and zeroes the counter before its launch, so calls must not overlap
// on the GPU (issue them on one stream, or order them) -- overlapping calls
// race on the table and the counter.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "kdgr_internal.h"
#include "scene.h"

namespace kdgr {
namespace {

constexpr int kNoAllocMaxViews = 256;
constexpr size_t kTableBytes = kNoAllocMaxViews * sizeof(ViewDesc);  // 24576
constexpr size_t kCounterOffset = (kTableBytes + 255) & ~size_t(255);
constexpr size_t kScratchBytes = 32 * 1024;
static_assert(kCounterOffset + kQueueBytes <= kScratchBytes, "no-alloc scratch too small");
static_assert(kQueueBytes / sizeof(uint32_t) <= 256, "queue words are zeroed by one 256-thread block");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// The view table of one call, passed by value as kernel parameters.
struct StageParams {
  ViewDesc views[kNoAllocMaxViews];
  int32_t n_views;
};
static_assert(sizeof(StageParams) <= 32764, "kernel parameters are limited to 32,764 bytes");

// Copies the call's views into the scratch table and zeroes the queue words.
__global__ void __launch_bounds__(256) k_noalloc_stage(const __grid_constant__ StageParams p) {
  ViewDesc* table = reinterpret_cast<ViewDesc*>(g_noalloc_scratch);
  uint32_t* queue = reinterpret_cast<uint32_t*>(g_noalloc_scratch + kCounterOffset);
  const int i = threadIdx.x;
  if (i < p.n_views) table[i] = p.views[i];
  if (i < (int)(kQueueBytes / sizeof(uint32_t))) queue[i] = 0u;
}

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_addr[kMaxDevices] = {nullptr};

// Device address of the scratch array on the current device (set up once).
cudaError_t scratch_address(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_addr[dev] = p;
  }
  *out = g_addr[dev];
  return cudaSuccess;
}

}  // namespace
}  // namespace kdgr

using namespace kdgr;

extern "C" int kdgr_render_batch_noalloc(kdgr_scene_t s, const kdgr_view* views, int n_views, float* rgb,
                                         float* alpha, float* depth, const kdgr_batch_config* cfg, void* stream) {
  static const char* kWho = "kdgr_render_batch_noalloc";
  if (!s || !views || n_views <= 0 || !rgb) {
    set_error(std::string(kWho) + ": null scene/views/output or no views");
    return KDGR_ERR_INVALID_ARG;
  }
  if (n_views > kNoAllocMaxViews) {
    set_error(std::string(kWho) + ": " + std::to_string(n_views) + " views exceed the fixed scratch limit of " +
              std::to_string(kNoAllocMaxViews) + " views");
    return KDGR_ERR_LIMIT;
  }
  kdgr_batch_config c;
  if (cfg) c = *cfg;
  else kdgr_batch_config_default(&c);
  int rc = check_batch_config(s, c);
  if (rc != KDGR_OK) {
    set_error(std::string(kWho) + ": " + kdgr_last_error());
    return rc;
  }
  StageParams p;
  p.n_views = n_views;
  uint32_t totals[3] = {0, 0, 0};
  rc = fill_view_table(views, n_views, p.views, totals);
  if (rc != KDGR_OK) {
    set_error(std::string(kWho) + ": " + kdgr_last_error());
    return rc;
  }
  DeviceScope on(s->device);
  if (on.err != cudaSuccess) return cuda_fail(on.err, "kdgr_render_batch_noalloc: cudaSetDevice");
  void* base = nullptr;
  cudaError_t e = scratch_address(&base);
  if (e != cudaSuccess) return cuda_fail(e, "kdgr_render_batch_noalloc: scratch address");
  ViewDesc* d_views = static_cast<ViewDesc*>(base);
  uint32_t* d_queue = reinterpret_cast<uint32_t*>(static_cast<unsigned char*>(base) + kCounterOffset);
  const cudaStream_t st = (cudaStream_t)stream;
  k_noalloc_stage<<<1, 256, 0, st>>>(p);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = launch_batch(s, c, d_views, n_views, totals, rgb, alpha, depth, d_queue, st);
  if (e != cudaSuccess) return cuda_fail(e, "kdgr_render_batch_noalloc");
  return KDGR_OK;
}
